// Device-resident particle system: simpleModel state + neighbour structure + pair force + updater.
//
// One timestep is the reference's simulation::performTimestep (src/simulation/simulation.cpp:84-95) with
//   velocityVerletNVE::performUpdate  (src/updaters/velocityVerletNVE.cpp:3-29):
//       disp = dt v + dt^2/2 f ; v += dt/2 f ; move (transport v) ; forces ; v += dt/2 f
//   noseHooverNVT::performUpdate      (src/updaters/noseHooverNVT.cpp:42-139):
//       chain ; v *= s ; move(dt/2 v) ; forces ; v += dt f, KE ; move(dt/2 v) ; chain ; v *= s
// where "forces" is simulation::computeForces -> force::computeForces -> simpleModel::findNeighbors
// (src/forces/baseForce.cpp:12-28, src/models/simpleModel.cpp:68-112) and "move" is simpleModel::moveParticles
// (src/models/simpleModel.cpp:44-66).  All of it stays on the device: the Nose-Hoover chain scalars live in device
// memory and are advanced by a one-thread kernel, the kinetic energy is reduced in a fixed order, and the cell list
// (hyperRectangularCellList::sort, src/utility/hyperRectangularCellList.cpp:82-125) is a stable counting sort.
// A step is a fixed kernel sequence, so it can be captured once as a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <math_constants.h>

#include "cssg_internal.cuh"

namespace {

constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 8;  // per thread
constexpr int KE_BLOCK = 256;

// ---- exclusive scan over int counts (total written at out[n]) -------------------------------------------------
__global__ void scan_local(const int* __restrict__ in, int n, int* __restrict__ out, int* __restrict__ blockSums)
{
    __shared__ int s[SCAN_BLOCK];
    const int base = blockIdx.x * SCAN_BLOCK * SCAN_ITEMS + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int sum = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        int i = base + k;
        v[k] = i < n ? in[i] : 0;
        sum += v[k];
    }
    s[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < SCAN_BLOCK; o <<= 1) {
        int t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    int run = s[threadIdx.x] - sum;
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        int i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (threadIdx.x == SCAN_BLOCK - 1) blockSums[blockIdx.x] = s[threadIdx.x];
}

__global__ void scan_blocks(int* blockSums, int nb, int* total)
{
    __shared__ int s[1024];
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += 1024) {
        int i = b0 + threadIdx.x;
        int v = i < nb ? blockSums[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            int t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) blockSums[i] = carry + s[threadIdx.x] - v;
        int last = s[1023];
        __syncthreads();
        carry += last;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void scan_add(int* out, int n, const int* blockSums)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += blockSums[i / (SCAN_BLOCK * SCAN_ITEMS)];
}

// ---- cell list (one grid per system, concatenated) -------------------------------------------------------------
__global__ void cell_assign(int n, const double* __restrict__ pos, const SysDesc* __restrict__ sys,
                            const int* __restrict__ sysOf, int* __restrict__ cellOf, int* __restrict__ count)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SysDesc& D = sys[sysOf ? sysOf[i] : 0];
    int ci[3];
    for (int c = 0; c < 3; ++c) {
        int q = (int)floor((pos[3 * i + c] - D.lo[c]) / D.cs[c]);
        ci[c] = max(0, min(D.nc[c] - 1, q));
    }
    int cell = D.cellBase + ci[0] + D.nc[0] * (ci[1] + D.nc[1] * ci[2]);
    cellOf[i] = cell;
    atomicAdd(&count[cell], 1);
}

__global__ void cell_scatter(int n, const int* __restrict__ cellOf, const int* __restrict__ start,
                             int* __restrict__ cursor, int* __restrict__ list, int* __restrict__ slotOf)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cellOf[i];
    int p = atomicAdd(&cursor[c], 1);
    list[start[c] + p] = i;
    slotOf[i] = p;
}

// stable order inside each occupied cell: particle index ascending (the order the reference's sort inserts them);
// the particle that landed in slot 0 of its cell sorts that cell
__global__ void cell_sort(int n, const int* __restrict__ cellOf, const int* __restrict__ start,
                          const int* __restrict__ slotOf, int* __restrict__ list)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || slotOf[i] != 0) return;
    int c = cellOf[i];
    int a = start[c], b = start[c + 1];
    for (int p = a + 1; p < b; ++p) {
        int x = list[p];
        int q = p - 1;
        while (q >= a && list[q] > x) {
            list[q + 1] = list[q];
            --q;
        }
        list[q + 1] = x;
    }
}

// ---- integrators ------------------------------------------------------------------------------------------------
// One thread per system: noseHooverNVT::propagateChain.  Chain k occupies len = 4 (M+1) + 2 doubles:
// (M+1) x {pos, vel, accel, mass}, then kineticEnergy, scale.
__global__ void nh_chain(double* chains, int K, int Mc, double T, double dt)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    double* bv = chains + (size_t)k * (4 * (Mc + 1) + 2);
    double& KE = bv[4 * (Mc + 1)];
    double& scale = bv[4 * (Mc + 1) + 1];
    const double dt2 = 0.5 * dt, dt4 = 0.25 * dt, dt8 = 0.125 * dt;
    double ef = 0;
    for (int ii = Mc - 1; ii > 0; --ii) {
        bv[4 * ii + 2] = (bv[4 * (ii - 1) + 3] * bv[4 * (ii - 1) + 1] * bv[4 * (ii - 1) + 1] - T) / bv[4 * ii + 3];
        ef = exp(-dt8 * bv[4 * (ii + 1) + 1]);
        bv[4 * ii + 1] *= ef;
        bv[4 * ii + 1] += bv[4 * ii + 2] * dt4;
        bv[4 * ii + 1] *= ef;
    }
    bv[2] = (2.0 * KE / bv[3] - 1.0);
    ef = exp(-dt8 * bv[5]);
    bv[1] *= ef;
    bv[1] += bv[2] * dt4;
    bv[1] *= ef;
    for (int ii = 0; ii < Mc; ++ii) bv[4 * ii] += dt2 * bv[4 * ii + 1];
    scale = exp(-dt2 * bv[1]);
    KE = scale * scale * KE;
    bv[2] = (2.0 * KE / bv[3] - 1.0);
    ef = exp(-dt8 * bv[5]);
    bv[1] *= ef;
    bv[1] += bv[2] * dt4;
    bv[1] *= ef;
    for (int ii = 1; ii < Mc; ++ii) {
        bv[4 * ii + 2] = (bv[4 * (ii - 1) + 3] * bv[4 * (ii - 1) + 1] * bv[4 * (ii - 1) + 1] - T) / bv[4 * ii + 3];
        ef = exp(-dt8 * bv[4 * (ii + 1) + 1]);
        bv[4 * ii + 1] *= ef;
        bv[4 * ii + 1] += bv[4 * ii + 2] * dt4;
        bv[4 * ii + 1] *= ef;
    }
}

__global__ void nvt_scale(int n, double* __restrict__ v, const double* __restrict__ chains, int Mc,
                          const int* __restrict__ sysOf, double* __restrict__ disp, double dt2)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    int k = sysOf ? sysOf[i / 3] : 0;
    double s = chains[(size_t)k * (4 * (Mc + 1) + 2) + 4 * (Mc + 1) + 1];
    v[i] = s * v[i];
    if (disp) disp[i] = dt2 * v[i];
}

__global__ void nvt_kick(int n, double* __restrict__ v, const double* __restrict__ f, double* __restrict__ disp,
                         double dt, double dt2, double* __restrict__ ke)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double vv[3];
    for (int c = 0; c < 3; ++c) {
        vv[c] = v[3 * i + c] + (dt / 1.0) * f[3 * i + c];
        v[3 * i + c] = vv[c];
        disp[3 * i + c] = dt2 * vv[c];
    }
    ke[i] = 0.5 * 1.0 * (vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
}

// one block per system: kinetic energy in a fixed summation order, written into that system's chain
__global__ void __launch_bounds__(KE_BLOCK) ke_reduce(const double* __restrict__ ke, const int* __restrict__ partBase,
                                                      double* chains, int Mc)
{
    __shared__ double sm[KE_BLOCK];
    int k = blockIdx.x;
    int a = partBase[k], b = partBase[k + 1];
    double acc = 0;
    for (int i = a + threadIdx.x; i < b; i += KE_BLOCK) acc += ke[i];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int o = KE_BLOCK / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) chains[(size_t)k * (4 * (Mc + 1) + 2) + 4 * (Mc + 1)] = sm[0];
}

// candidate rows -> CSR pairs (pi, pj); rows longer than the row capacity are truncated and reported
__global__ void compact_pairs(int n, int cap, const int* __restrict__ count, const int* __restrict__ off,
                              const int* __restrict__ candJ, int* __restrict__ pi, int* __restrict__ pj)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = count[i], o = off[i];
    for (int q = 0; q < c; ++q) {
        pi[o + q] = i;
        pj[o + q] = candJ[(size_t)i * cap + q];
    }
}

// rows longer than the row capacity cannot be screened: clamp them and report a capacity failure
__global__ void clamp_counts(int n, int cap, int* __restrict__ count, int* __restrict__ statusBits)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && count[i] > cap) {
        count[i] = cap;
        atomicOr(statusBits, 1 << CSSG_ST_CAPACITY);
    }
}

__global__ void count_screened(int m, const int* __restrict__ total, const unsigned char* __restrict__ skip,
                               unsigned long long* __restrict__ out)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int nP = *total;
    int a = p < nP ? 1 : 0, b = (p < nP && skip[p]) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0 && a) {
        atomicAdd(&out[0], (unsigned long long)a);
        atomicAdd(&out[1], (unsigned long long)b);
    }
    (void)m;
}

}  // namespace

struct cssg_system {
    cssg_ctx* ctx;
    int K = 1;             // independent systems
    int n = 0;             // particles over all systems
    cssg_params P;         // shared integrator parameters (systems' own force/patch parameters live in hsys)
    std::vector<const cssg_mesh*> meshes;
    std::vector<cssg_params> params;
    std::vector<int> partBase;  // K + 1
    std::vector<SysDesc> hsys;
    SysDesc* dsys = nullptr;
    SysDesc* dsysScreen = nullptr;  // the same systems with the screened-CSR search mode
    DevMesh* dmeshes = nullptr;
    int* sysOf = nullptr;       // per particle (null when K == 1)
    int* dPartBase = nullptr;
    // state
    int* face = nullptr;
    double* bary = nullptr;
    double* vel = nullptr;
    double* force = nullptr;
    double* disp = nullptr;
    double* pos = nullptr;
    int* walkStatus = nullptr;
    int* srcStatus = nullptr;
    int* statusBits = nullptr;               // device: OR of 1 << status over walks and sources
    unsigned long long* counters = nullptr;  // device: crossings, windows, launches, in-range pairs, capacity hits
    // cell list
    bool useCells = false;
    int totalCells = 0;
    int* cellOf = nullptr;
    int* cellCount = nullptr;
    int* cellStart = nullptr;
    int* cellCursor = nullptr;
    int* cellList = nullptr;
    int* slotOf = nullptr;
    int* scanBlocks = nullptr;
    int nScanBlocks = 0;
    // geodesic scratch of the three passes: regular (tables in shared memory when they fit), medium (sources of
    // large-patch systems and regular overflows, many warps) and large (medium overflows, one warp per SM)
    GeoCaps caps, midCaps, bigCaps;
    void* scratch = nullptr;
    void* midScratch = nullptr;
    void* bigScratch = nullptr;
    size_t slotBytes = 0, midSlotBytes = 0, bigSlotBytes = 0;
    int nSlots = 0, nMidSlots = 0, nBigSlots = 0;
    // [0] regular work counter, [1] medium work counter, [2] medium item count, [3] large work counter,
    // [4] large item count
    int* work = nullptr;
    int* failList = nullptr;   // sources for the medium pass
    int* failList2 = nullptr;  // sources for the large pass
    // pair output
    int pairCap = 0;
    double* pairD = nullptr;
    double* pairT = nullptr;
    int* pairJ = nullptr;
    int* pairCount = nullptr;
    // learned screen (candidate lists -> features -> tensor-core MLP -> screened CSR propagation)
    bool screen = false;
    double margin = 0;
    float* mlpParams = nullptr;
    int candCap = 0;
    int* candJPad = nullptr;     // n x candCap
    int* candCount = nullptr;    // n (+1 for the scan total)
    double* maxChord = nullptr;  // n
    int* candOff = nullptr;      // n + 1
    int* pairI = nullptr;        // n x candCap (compact prefix used)
    int* pairJc = nullptr;
    void* X = nullptr;           // n x candCap x 16 BF16
    float* chordS = nullptr;
    float* yhat = nullptr;
    unsigned char* skip = nullptr;
    int* candScanBlocks = nullptr;
    int nCandScanBlocks = 0;
    int* mlpErr = nullptr;
    unsigned long long* screenCounters = nullptr;  // [0] candidate pairs, [1] screened out
    // regular pass with one source per lane (lanes.cu): lanes per warp (0: the source-group kernel), per-lane
    // capacities, scratch of nLaneWarps warps
    int laneLanes = 0;
    int laneSplit = 0;  // with the lane pass: the costliest sources (by the last evaluation) that the group pass takes
    int tuneMidGroup = 0, tuneBigGroup = 0;  // warps per source of the medium and large passes (0: the regular pass's)
    bool patchSystems = false;  // every system: reference patches and cell-list candidates (search mode 1 or 3)
    LaneCaps laneCaps{};
    void* laneScratch = nullptr;
    int nLaneWarps = 0;
    // periodic exact audit of the screen: every auditEvery-th step runs the screened and the exact force passes on
    // the same positions (the exact one drives the step) and compares the in-range pair counts per source
    int auditEvery = 0;
    long long stepsDone = 0;                       // steps since the audit schedule was set
    bool auditStep = false;                        // the step being launched or captured is an audit step
    double* forceAudit = nullptr;                  // n x 3: the screened pass's forces in an audit step
    int* inRangeScr = nullptr;                     // n: in-range pairs per source, screened pass
    int* inRangeExact = nullptr;                   // n: the same, exact pass
    int* screenOff = nullptr;                      // device flag: an audit found a dropped pair; nothing is skipped
    unsigned long long* auditCounters = nullptr;   // [0] audits run, [1] sources that lost an in-range pair
    // FIRE minimisation (device state, transport buffer, reduction partials) and stress partials
    void* fireState = nullptr;
    double* fireTrans = nullptr;  // n x 2 x 3: force and velocity carried by the walk
    int* fireDone = nullptr;      // K + 1: per-system stop flags, then "every system stopped"
    double* stressPartials = nullptr;
    // NVT
    double* chains = nullptr;
    double* ke = nullptr;
    // graph
    cudaGraphExec_t graphExec = nullptr;
    cudaGraphExec_t graphAudit = nullptr;  // the audit step's graph (screen with periodic audit)
    double delta = 1e300;  // bucket width of the propagation order (distance-banded rounds)
    // tuning (cssg_system_autotune / cssg_system_set_tuning): band width scale, warps per block, medium-pass slots
    double tuneDelta = 1.0;
    int tuneWpb = 8;
    int tuneWarpsPerSM = 0;  // 0: every slot
    int tuneGroup = 1;       // warps per source (1, 2, 4, 8)
    int tuneWide = 0;        // kernel build: bit 0 = up to 255 registers, bit 1 = out-of-line hash-table probes
    bool tuneLpt = false;    // sources in decreasing order of their last cost (longest first) instead of cell order
    int* srcCost = nullptr;  // n: work of each source in the last force evaluation
    int* lptOrder = nullptr; // n
    int* lptBuckets = nullptr;  // 64: bucket counts, then cursors
    int midSlotsMax = 0;  // allocated medium slots; the launch uses nMidSlots <= midSlotsMax
    int maxWindows = 0, midMaxWindows = 0, bigMaxWindows = 0;  // per-source work caps of the three passes
    // timing
    bool timing = false;
    std::vector<cudaEvent_t> events;
    int eventsUsed = 0;
};

namespace {

int alloc(void** p, size_t bytes)
{
    CSSG_CUDA(cudaMalloc(p, bytes ? bytes : 16));
    return CSSG_OK;
}

int chain_len(const cssg_system* s) { return 4 * (std::max(1, s->P.chain_length) + 1) + 2; }

int record(cssg_system* s)
{
    if (!s->timing) return -1;
    if (s->eventsUsed >= (int)s->events.size()) return -1;
    int k = s->eventsUsed++;
    cudaEventRecord(s->events[k], s->ctx->stream);
    return k;
}

// ---- longest-processing-time-first order of the sources (by the last evaluation's cost) -----------------------
__device__ __forceinline__ int cost_bucket(int c)
{
    // 32 buckets by log2(cost), largest cost first
    const int lg = 31 - __clz(max(c, 1));
    return 31 - min(31, lg);
}

__global__ void lpt_count(int n, const int* __restrict__ cost, int* __restrict__ buckets)
{
    __shared__ int local[32];
    if (threadIdx.x < 32) local[threadIdx.x] = 0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&local[cost_bucket(cost[i])], 1);
    __syncthreads();
    if (threadIdx.x < 32 && local[threadIdx.x]) atomicAdd(&buckets[threadIdx.x], local[threadIdx.x]);
}

__global__ void lpt_scan(int* buckets)
{
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int b = 0; b < 32; ++b) {
            buckets[32 + b] = acc;
            acc += buckets[b];
        }
    }
}

__global__ void lpt_scatter(int n, const int* __restrict__ order, const int* __restrict__ cost, int* buckets,
                            int* __restrict__ out)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int si = order ? order[k] : k;
    out[atomicAdd(&buckets[32 + cost_bucket(cost[si])], 1)] = si;
}

// the three passes above in one block, for source counts one block sorts quickly
constexpr int kLptSmallMax = 16384;
__global__ void __launch_bounds__(1024) lpt_small(int n, const int* __restrict__ order, const int* __restrict__ cost,
                                                   int* __restrict__ out)
{
    __shared__ int count[32], cursor[32];
    if (threadIdx.x < 32) count[threadIdx.x] = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) atomicAdd(&count[cost_bucket(cost[order ? order[k] : k])], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int b = 0; b < 32; ++b) {
            cursor[b] = acc;
            acc += count[b];
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int si = order ? order[k] : k;
        out[atomicAdd(&cursor[cost_bucket(cost[si])], 1)] = si;
    }
}

// the padded candidate rows of the cell-list search (learned screen and one-source-per-lane pass)
int ensure_candidate_rows(cssg_system* s)
{
    if (s->candJPad) return CSSG_OK;
    const int n = s->n;
    s->candCap = std::max(32, 2 * s->caps.CT);
    int rc;
    if ((rc = alloc((void**)&s->candJPad, sizeof(int) * (size_t)n * s->candCap)) ||
        (rc = alloc((void**)&s->candCount, sizeof(int) * (n + 1))) || (rc = alloc((void**)&s->maxChord, sizeof(double) * n)))
        return rc;
    return CSSG_OK;
}

// switches the regular pass to one source per lane (16 or 32 lanes per warp) or back to source groups (0); the
// lane scratch is allocated on first use
int set_lanes(cssg_system* s, int lanes)
{
    if (lanes > 0 && !s->useCells) {
        cssg_set_error("cssg_system_set_lanes: the one-source-per-lane pass needs the cell-list neighbour structure");
        return CSSG_ERR_ARG;
    }
    if (lanes > 0 && !s->laneScratch) {
        if (int rc = ensure_candidate_rows(s)) return rc;
        // per-lane tables from the regular pass's estimates: targets up to the candidate row, face and vertex tables at
        // half the regular tables' margins (a lane's tables hold one source), live windows up to twice the face table
        LaneCaps& c = s->laneCaps;
        c.CT = std::min(s->candCap, std::max(16, s->caps.CT));
        c.CF = std::max(64, s->caps.CF / 2);
        c.CV = std::max(64, s->caps.CV / 2);
        c.CW = std::max(64, std::min(s->caps.CW, c.CF * 2));
        int sms = 0;
        CSSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->ctx->device));
        const long long batches = (s->n + 15) / 16;
        s->nLaneWarps = (int)std::max<long long>(1, std::min<long long>(batches, (long long)sms * 16));
        if (int rc = alloc(&s->laneScratch, cssg_lane_warp_bytes(c) * (size_t)s->nLaneWarps)) return rc;
    }
    s->laneLanes = lanes;
    return CSSG_OK;
}

// Longest-first within spatial segments (the one-source-per-lane pass): the cell order is cut into segments of 256
// sources and each segment is sorted by the last evaluation's cost, largest first (bitonic sort in shared memory).
// Consecutive sources, which a warp takes together, then cost about the same and still lie close on the mesh.
__global__ void __launch_bounds__(256) lpt_segmented(int n, const int* __restrict__ order, const int* __restrict__ cost,
                                                     int* __restrict__ out)
{
    __shared__ int kc[256], kv[256];
    const int i = threadIdx.x, g = blockIdx.x * 256 + i;
    const int si = g < n ? (order ? order[g] : g) : -1;
    kc[i] = g < n ? cost[si] : -1;  // padding sorts last
    kv[i] = si;
    __syncthreads();
    for (int k = 2; k <= 256; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int p = i ^ j;
            if (p > i) {
                const int a = kc[i], b = kc[p];
                if ((i & k) == 0 ? a < b : a > b) {
                    kc[i] = b;
                    kc[p] = a;
                    const int t = kv[i];
                    kv[i] = kv[p];
                    kv[p] = t;
                }
            }
            __syncthreads();
        }
    if (g < n) out[g] = kv[i];
}

// findNeighbors + computeForces into forceOut; kick: the velocity-Verlet second half kick of every particle is
// applied where its force is written (velocityVerletNVE.cpp:23-29); useScreen: the learned-screen path (else the
// exact one); inRangeOut (nullable): in-range pairs per source; cells: rebuild the cell list first
void launch_forces_ex(cssg_system* s, bool kick, bool useScreen, double* forceOut, int* inRangeOut, bool cells)
{
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    const int tb = 256;
    if (s->useCells && cells) {
        cudaMemsetAsync(s->cellCount, 0, sizeof(int) * (s->totalCells + 1), st);
        cudaMemsetAsync(s->cellCursor, 0, sizeof(int) * s->totalCells, st);
        cell_assign<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->pos, s->dsys, s->sysOf, s->cellOf, s->cellCount);
        scan_local<<<s->nScanBlocks, SCAN_BLOCK, 0, st>>>(s->cellCount, s->totalCells, s->cellStart, s->scanBlocks);
        scan_blocks<<<1, 1024, 0, st>>>(s->scanBlocks, s->nScanBlocks, s->cellStart + s->totalCells);
        scan_add<<<(s->totalCells + 255) / 256, 256, 0, st>>>(s->cellStart, s->totalCells, s->scanBlocks);
        cell_scatter<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->cellOf, s->cellStart, s->cellCursor, s->cellList,
                                                       s->slotOf);
        cell_sort<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->cellOf, s->cellStart, s->slotOf, s->cellList);
    }
    cudaMemsetAsync(s->work, 0, 6 * sizeof(int), st);
    GeoLaunch L;
    memset(&L, 0, sizeof(L));
    L.sys = useScreen ? s->dsysScreen : s->dsys;
    L.sysOf = s->sysOf;
    L.nSrc = n;
    L.srcFace = s->face;
    L.srcBary = s->bary;
    L.srcPos = s->pos;
    L.order = s->useCells ? s->cellList : nullptr;
    L.partFace = s->face;
    L.partBary = s->bary;
    L.partPos = s->pos;
    L.cellStart = s->cellStart;
    L.cellList = s->cellList;
    L.dOut = s->pairD;
    L.tsOut = s->pairT;
    L.pairJ = s->pairJ;
    L.pairCount = s->pairCount;
    L.pairCap = s->pairCap;
    L.force = forceOut;
    L.inRangeOut = inRangeOut;
    L.status = s->srcStatus;
    L.statusBits = s->statusBits;
    L.kickVel = kick ? s->vel : nullptr;
    L.kickDt = s->P.dt;
    L.counters = s->counters + 1;
    L.delta = s->delta;
    L.maxRounds = 4096;
    L.maxWindows = s->maxWindows;
    L.caps = s->caps;
    L.scratch = s->scratch;
    L.slotBytes = s->slotBytes;
    L.nSlots = s->nSlots;
    L.workCounter = s->work;
    L.failList = s->failList;
    L.failCount = s->work + 2;
    L.routeBig = 1;
    L.deltaScale = s->tuneDelta;
    L.wpbMax = s->tuneWpb;
    L.warpsPerSM = s->tuneWarpsPerSM;
    L.groupWarps = s->tuneGroup;
    L.wideRegs = s->tuneWide & 1;
    L.hashOutline = (s->tuneWide >> 1) & 1;
    L.patchSystems = s->patchSystems ? 1 : 0;
    L.srcCost = s->srcCost;
    L.device = s->ctx->device;
    // split of the regular pass: the costliest sources go to the source-group pass, the rest to the lane pass (the
    // global longest-first order picks them)
    const int split = s->laneLanes > 0 ? std::min(n, s->laneSplit) : 0;
    if (s->tuneLpt && s->laneLanes > 0 && split == 0) {
        lpt_segmented<<<(n + 255) / 256, 256, 0, st>>>(n, L.order, s->srcCost, s->lptOrder);
        L.order = s->lptOrder;
    } else if (s->tuneLpt || split > 0) {
        if (n <= kLptSmallMax) {
            lpt_small<<<1, 1024, 0, st>>>(n, L.order, s->srcCost, s->lptOrder);
        } else {
            cudaMemsetAsync(s->lptBuckets, 0, 64 * sizeof(int), st);
            lpt_count<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->srcCost, s->lptBuckets);
            lpt_scan<<<1, 32, 0, st>>>(s->lptBuckets);
            lpt_scatter<<<(n + tb - 1) / tb, tb, 0, st>>>(n, L.order, s->srcCost, s->lptBuckets, s->lptOrder);
        }
        L.order = s->lptOrder;
    }
    if (useScreen) {
        // learned screen: candidate rows -> CSR pairs -> features -> tensor-core MLP -> skip flags; the propagation
        // then reads the CSR (screened pairs keep their faces in the patch but are not queried)
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->ctx->device);
        cssg_launch_candidates(L, n, s->candCap, s->candJPad, s->candCount, s->maxChord, st);
        clamp_counts<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->candCap, s->candCount, s->statusBits);
        scan_local<<<s->nCandScanBlocks, SCAN_BLOCK, 0, st>>>(s->candCount, n, s->candOff, s->candScanBlocks);
        scan_blocks<<<1, 1024, 0, st>>>(s->candScanBlocks, s->nCandScanBlocks, s->candOff + n);
        scan_add<<<(n + 255) / 256, 256, 0, st>>>(s->candOff, n, s->candScanBlocks);
        compact_pairs<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->candCap, s->candCount, s->candOff, s->candJPad,
                                                        s->pairI, s->pairJc);
        cssg_launch_screen(s->dsysScreen, s->sysOf, n * s->candCap, s->candOff + n, s->pairI, s->pairJc, s->face,
                           s->pos, s->X, s->chordS, s->mlpParams, s->yhat, s->skip, s->margin, s->mlpErr, sms, st,
                           s->screenOff);
        count_screened<<<(n * s->candCap + 255) / 256, 256, 0, st>>>(n * s->candCap, s->candOff + n, s->skip,
                                                                    s->screenCounters);
        L.candOff = s->candOff;
        L.candJ = s->pairJc;
        L.candSkip = s->skip;
        L.threshold = s->maxChord;
    }
    record(s);
    if (s->laneLanes > 0) {
        // regular pass with one source per lane; without the screen it reads the cell-list candidates as padded rows
        if (!useScreen) {
            cssg_launch_candidates(L, n, s->candCap, s->candJPad, s->candCount, s->maxChord, st);
            L.rowJ = s->candJPad;
            L.rowCount = s->candCount;
            L.rowChord = s->maxChord;
            L.rowCap = s->candCap;
        }
        if (split > 0) {
            // the costliest sources with source groups (their windows fill a group's lanes)
            GeoLaunch G = L;
            G.nSrc = split;
            cssg_launch_geodesic(G, st);
        }
        GeoLaunch LL = L;
        LL.order = L.order + split;
        LL.nSrc = n - split;
        LL.workCounter = s->work + 5;
        LL.scratch = s->laneScratch;
        LL.nSlots = s->nLaneWarps;
        cssg_launch_lanes(LL, s->laneCaps, s->laneLanes, st);
    } else {
        cssg_launch_geodesic(L, st);
    }
    // medium pass: sources of large-patch systems and regular-pass overflows (exits at once when there are none)
    GeoLaunch R = L;
    R.caps = s->midCaps;
    R.scratch = s->midScratch;
    R.slotBytes = s->midSlotBytes;
    R.nSlots = s->nMidSlots;
    R.workCounter = s->work + 1;
    R.order = s->failList;
    R.itemCountDev = s->work + 2;
    R.failList = s->failList2;
    R.failCount = s->work + 4;
    R.routeBig = 0;
    R.warpsPerSM = 0;
    R.maxRounds = 1 << 15;
    R.maxWindows = s->midMaxWindows;
    if (s->tuneMidGroup) R.groupWarps = s->tuneMidGroup;
    cssg_launch_geodesic(R, st);
    // large pass: medium-pass overflows
    GeoLaunch B = R;
    B.caps = s->bigCaps;
    B.scratch = s->bigScratch;
    B.slotBytes = s->bigSlotBytes;
    B.nSlots = s->nBigSlots;
    B.workCounter = s->work + 3;
    B.order = s->failList2;
    B.itemCountDev = s->work + 4;
    B.failList = nullptr;
    B.failCount = nullptr;
    B.maxWindows = s->bigMaxWindows;
    B.groupWarps = s->tuneBigGroup ? s->tuneBigGroup : L.groupWarps;
    cssg_launch_geodesic(B, st);
    record(s);
}

void launch_forces(cssg_system* s, bool kick = false)
{
    launch_forces_ex(s, kick, s->screen, s->force, nullptr, true);
}

// Audit of the screen: sources whose screened pass found fewer in-range pairs than the exact pass on the same
// positions (the screen dropped an in-range pair) are counted, and any such source switches the screen off on the
// device (screen_decide then keeps every pair).
__global__ void audit_compare(int n, const int* __restrict__ scr, const int* __restrict__ exact,
                              unsigned long long* counters, int* off)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool lost = i < n && scr[i] < exact[i];
    const unsigned m = __ballot_sync(0xffffffffu, lost);
    if ((threadIdx.x & 31) == 0 && m) {
        atomicAdd(&counters[1], (unsigned long long)__popc(m));
        atomicExch(off, 1);
    }
    if (i == 0) atomicAdd(&counters[0], 1ull);
}

// the force evaluation of one step: the plain one, or on an audit step the screened pass (into scratch) and the
// exact pass (which drives the step), then their comparison
void launch_step_forces(cssg_system* s, bool kick)
{
    if (!(s->screen && s->auditStep)) {
        launch_forces(s, kick);
        return;
    }
    const int n = s->n;
    launch_forces_ex(s, false, true, s->forceAudit, s->inRangeScr, true);
    launch_forces_ex(s, kick, false, s->force, s->inRangeExact, false);
    audit_compare<<<(n + 255) / 256, 256, 0, s->ctx->stream>>>(n, s->inRangeScr, s->inRangeExact, s->auditCounters,
                                                               s->screenOff);
}

// moveParticles with the velocity transported; kick: the velocity-Verlet first half (disp = dt v + dt^2 f / 2,
// v += dt f / 2, velocityVerletNVE.cpp:14-21) is done by the walk kernel itself
void launch_walk(cssg_system* s, bool kick = false)
{
    cudaStream_t st = s->ctx->stream;
    record(s);
    cssg_launch_transport(s->dmeshes, s->sysOf, s->n, s->face, s->bary, s->disp, s->vel, 1, s->walkStatus,
                          s->counters, s->pos, st, nullptr, s->statusBits, kick ? s->force : nullptr, s->P.dt);
    record(s);
}

void launch_step(cssg_system* s)
{
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    const int tb = 256;
    const double dt = s->P.dt;
    if (s->P.integrator == 0) {
        // velocityVerletNVE::performUpdate (velocityVerletNVE.cpp:3-29): first half kick + drift inside the walk
        // kernel, second half kick where each force is written
        launch_walk(s, true);
        launch_step_forces(s, true);
    } else {
        const int Mc = s->P.chain_length;
        const double T = s->P.temperature;
        const int K = s->K;
        nh_chain<<<(K + 63) / 64, 64, 0, st>>>(s->chains, K, Mc, T, dt);
        nvt_scale<<<(3 * n + tb - 1) / tb, tb, 0, st>>>(n, s->vel, s->chains, Mc, s->sysOf, s->disp, 0.5 * dt);
        launch_walk(s);
        launch_step_forces(s, false);
        nvt_kick<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->vel, s->force, s->disp, dt, 0.5 * dt, s->ke);
        ke_reduce<<<K, KE_BLOCK, 0, st>>>(s->ke, s->dPartBase, s->chains, Mc);
        launch_walk(s);
        nh_chain<<<(K + 63) / 64, 64, 0, st>>>(s->chains, K, Mc, T, dt);
        nvt_scale<<<(3 * n + tb - 1) / tb, tb, 0, st>>>(n, s->vel, s->chains, Mc, s->sysOf, nullptr, 0.0);
    }
}

// noseHooverNVT::setBathVariables per system (its own particle count)
int reset_chain(cssg_system* s)
{
    int Mc = std::max(1, s->P.chain_length), len = chain_len(s);
    std::vector<double> h((size_t)len * s->K, 0.0);
    double T = s->P.temperature, tau = s->P.tau;
    for (int k = 0; k < s->K; ++k) {
        double* c = &h[(size_t)k * len];
        int nk = s->partBase[k + 1] - s->partBase[k];
        c[3] = 2.0 * (nk - 1) * T * tau * tau;
        for (int ii = 1; ii < Mc + 1; ++ii) c[4 * ii + 3] = T * tau * tau;
        c[4 * (Mc + 1)] = c[3];
        c[4 * (Mc + 1) + 1] = 1.0;
    }
    CSSG_CUDA(cudaMemcpyAsync(s->chains, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s->ctx->stream));
    CSSG_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return CSSG_OK;
}

int next_pow2_ll(long long x)
{
    int p = 1;
    while (p < x && p < (1 << 30)) p <<= 1;
    return p;
}

}  // namespace

extern "C" int cssg_system_create_batched(cssg_ctx* ctx, int K, const cssg_mesh* const* meshes, const int* counts,
                                          const cssg_params* params, cssg_system** out)
{
    if (!ctx || K <= 0 || !meshes || !counts || !params || !out) {
        cssg_set_error("cssg_system_create: bad arguments");
        return CSSG_ERR_ARG;
    }
    for (int k = 0; k < K; ++k) {
        const cssg_params& P = params[k];
        if (!meshes[k] || counts[k] <= 0 || P.integrator < 0 || P.integrator > 1 || P.force_kind < 0 ||
            P.force_kind > 1 || !(P.dt > 0) || (P.integrator == 1 && P.chain_length < 1) || !(P.cutoff > 0)) {
            cssg_set_error("cssg_system_create: bad parameters");
            return CSSG_ERR_ARG;
        }
        if (P.integrator != params[0].integrator || P.dt != params[0].dt || P.temperature != params[0].temperature ||
            P.tau != params[0].tau || P.chain_length != params[0].chain_length || (P.range > 0) != (params[0].range > 0)) {
            cssg_set_error("cssg_system_create: batched systems must share integrator, dt, T, tau, chain length and "
                           "neighbour structure kind");
            return CSSG_ERR_ARG;
        }
    }
    CSSG_CUDA(cudaSetDevice(ctx->device));
    cssg_system* s = new cssg_system();
    s->ctx = ctx;
    s->K = K;
    s->P = params[0];
    s->meshes.assign(meshes, meshes + K);
    s->params.assign(params, params + K);
    s->partBase.assign(K + 1, 0);
    for (int k = 0; k < K; ++k) s->partBase[k + 1] = s->partBase[k] + counts[k];
    const int n = s->n = s->partBase[K];
    int rc = CSSG_OK;
#define TRY(x)                      \
    if ((rc = (x)) != CSSG_OK) {    \
        cssg_system_destroy(s);     \
        return rc;                  \
    }
    TRY(alloc((void**)&s->face, sizeof(int) * n));
    TRY(alloc((void**)&s->bary, sizeof(double) * 3 * n));
    TRY(alloc((void**)&s->vel, sizeof(double) * 3 * n));
    TRY(alloc((void**)&s->force, sizeof(double) * 3 * n));
    TRY(alloc((void**)&s->disp, sizeof(double) * 3 * n));
    TRY(alloc((void**)&s->pos, sizeof(double) * 3 * n));
    TRY(alloc((void**)&s->walkStatus, sizeof(int) * n));
    TRY(alloc((void**)&s->srcStatus, sizeof(int) * n));
    TRY(alloc((void**)&s->statusBits, sizeof(int)));
    TRY(alloc((void**)&s->counters, sizeof(unsigned long long) * 8));
    TRY(alloc((void**)&s->work, sizeof(int) * 6));
    TRY(alloc((void**)&s->failList, sizeof(int) * n));
    TRY(alloc((void**)&s->failList2, sizeof(int) * n));
    TRY(alloc((void**)&s->srcCost, sizeof(int) * n));
    TRY(alloc((void**)&s->lptOrder, sizeof(int) * n));
    TRY(alloc((void**)&s->lptBuckets, sizeof(int) * 64));
    cudaMemset(s->srcCost, 0, sizeof(int) * n);
    TRY(alloc((void**)&s->ke, sizeof(double) * n));
    TRY(alloc((void**)&s->dPartBase, sizeof(int) * (K + 1)));
    cudaMemset(s->force, 0, sizeof(double) * 3 * n);
    cudaMemset(s->vel, 0, sizeof(double) * 3 * n);
    cudaMemset(s->face, 0, sizeof(int) * n);
    cudaMemset(s->statusBits, 0, sizeof(int));
    cudaMemset(s->counters, 0, sizeof(unsigned long long) * 8);
    cudaMemcpy(s->dPartBase, s->partBase.data(), sizeof(int) * (K + 1), cudaMemcpyHostToDevice);
    if (K > 1) {
        std::vector<int> so(n);
        for (int k = 0; k < K; ++k)
            for (int i = s->partBase[k]; i < s->partBase[k + 1]; ++i) so[i] = k;
        TRY(alloc((void**)&s->sysOf, sizeof(int) * n));
        cudaMemcpy(s->sysOf, so.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    }
    // per-system descriptors: mesh, interaction parameters, grid (hyperRectangularCellList::setGridSize: cells of
    // size >= range over the origin-including bounding box), particle and cell offsets
    s->useCells = params[0].range > 0;
    s->patchSystems = s->useCells;
    for (int k = 0; k < K; ++k) s->patchSystems = s->patchSystems && params[k].submesh != 0;
    long long cellTotal = 0;
    s->hsys.resize(K);
    std::vector<DevMesh> hm(K);
    long long maxF = 0, maxV = 0, maxT = 0;           // regular tables: systems whose patches fit shared memory
    long long bigF = 0, bigV = 0, bigT = 0;           // large tables: every system (retry and binned sources)
    const long long kRegularTable = 1024;             // entries per table that keep a warp's tables in ~20 KB
    bool anyBig = false;
    for (int k = 0; k < K; ++k) {
        const cssg_params& P = params[k];
        const cssg_mesh* m = meshes[k];
        SysDesc& D = s->hsys[k];
        memset(&D, 0, sizeof(D));
        D.mesh = m->d;
        hm[k] = m->d;
        D.searchMode = s->useCells ? 1 : 2;
        D.submesh = P.submesh;
        D.forceKind = P.force_kind;
        D.partBase = s->partBase[k];
        D.nPart = counts[k];
        D.range2 = P.range * P.range;
        D.maxDist = P.max_dist;
        D.cutoff = P.cutoff;
        D.k = P.k;
        D.sigma = P.sigma;
        D.delta = m->meanEdge;
        long long cells = 1;
        for (int c = 0; c < 3; ++c) {
            double ext = m->d.bbMax[c] - m->d.bbMin[c];
            D.lo[c] = m->d.bbMin[c];
            if (s->useCells) {
                D.nc[c] = std::max(1, (int)std::floor(ext / P.range));
                D.cs[c] = ext / D.nc[c];
            } else {
                D.nc[c] = 1;
                D.cs[c] = 1;
            }
            cells *= D.nc[c];
        }
        D.cellBase = (int)cellTotal;
        cellTotal += s->useCells ? cells : 0;
        if (cellTotal > (1LL << 28)) {
            cssg_set_error("cssg_system_create: cell grid too large for the interaction range");
            cssg_system_destroy(s);
            return CSSG_ERR_CAPACITY;
        }
        // table sizes from the expected neighbourhood: faces with a vertex within reach (patch radius <= range, or
        // the cutoff on the whole mesh) and candidates within the range
        double reach = P.cutoff;
        if (P.submesh && P.max_dist < reach) reach = P.max_dist;
        double rr = reach + m->meanEdge;
        long long estF = (long long)(1.3 * 3.14159265 * rr * rr / m->meanFaceArea) + 16;
        if (estF > m->d.nF) estF = m->d.nF;
        long long estV = std::min<long long>(m->d.nV, estF / 2 + 4 * (long long)std::sqrt((double)estF) + 16);
        double density = counts[k] / m->area;
        long long estT = P.range > 0 ? (long long)(density * 3.14159265 * P.range * P.range) : counts[k];
        estT = std::min<long long>(std::max<long long>(32, 4 * estT + 16), std::max(32, counts[k]));
        bigF = std::max(bigF, estF);
        bigV = std::max(bigV, estV);
        bigT = std::max(bigT, estT);
        if (next_pow2_ll(3 * (estF + estT) / 2 + 32) > kRegularTable || next_pow2_ll(2 * estV + 32) > kRegularTable) {
            D.bigBin = 1;
            anyBig = true;
        } else {
            maxF = std::max(maxF, estF);
            maxV = std::max(maxV, estV);
            maxT = std::max(maxT, estT);
        }
    }
    if (maxF == 0) {  // every system is large: the regular pass only routes sources to the large one
        maxF = 16;
        maxV = 16;
        maxT = 32;
    }
    {
        double me = 0;
        for (int k = 0; k < K; ++k) me = std::max(me, meshes[k]->meanEdge);
        s->delta = me;
    }
    TRY(alloc((void**)&s->dsys, sizeof(SysDesc) * K));
    TRY(alloc((void**)&s->dmeshes, sizeof(DevMesh) * K));
    cudaMemcpy(s->dsys, s->hsys.data(), sizeof(SysDesc) * K, cudaMemcpyHostToDevice);
    cudaMemcpy(s->dmeshes, hm.data(), sizeof(DevMesh) * K, cudaMemcpyHostToDevice);
    if (s->useCells) {
        s->totalCells = (int)cellTotal;
        s->nScanBlocks = (int)((cellTotal + SCAN_BLOCK * SCAN_ITEMS - 1) / (SCAN_BLOCK * SCAN_ITEMS));
        TRY(alloc((void**)&s->cellOf, sizeof(int) * n));
        TRY(alloc((void**)&s->cellCount, sizeof(int) * (cellTotal + 1)));
        TRY(alloc((void**)&s->cellStart, sizeof(int) * (cellTotal + 1)));
        TRY(alloc((void**)&s->cellCursor, sizeof(int) * cellTotal));
        TRY(alloc((void**)&s->cellList, sizeof(int) * n));
        TRY(alloc((void**)&s->slotOf, sizeof(int) * n));
        TRY(alloc((void**)&s->scanBlocks, sizeof(int) * (s->nScanBlocks + 1)));
    }
    s->caps.CT = (int)maxT;
    s->caps.CF = next_pow2_ll(3 * (maxF + s->caps.CT) / 2 + 32);
    s->caps.CV = next_pow2_ll(2 * maxV + 32);
    s->caps.CW = (int)(6 * maxF + 256);
    s->caps.CL = (int)(maxV + 64);
    s->caps.CLOG = (int)(4 * s->caps.CT + 2 * maxF + 128);
    // medium tables: the largest estimate of any system with the regular pass's margins, and never smaller than
    // 2x the regular tables
    s->midCaps.CT = (int)std::max<long long>(2LL * s->caps.CT, bigT);
    s->midCaps.CF = next_pow2_ll(std::max<long long>(2LL * s->caps.CF, 3 * (bigF + s->midCaps.CT) / 2 + 32));
    s->midCaps.CV = next_pow2_ll(std::max<long long>(2LL * s->caps.CV, 2 * bigV + 32));
    s->midCaps.CW = (int)std::max<long long>(2LL * s->caps.CW, 6 * bigF + 256);
    s->midCaps.CL = (int)std::max<long long>(2LL * s->caps.CL, bigV + 64);
    s->midCaps.CLOG = (int)std::max<long long>(2LL * s->caps.CLOG, 4 * s->midCaps.CT + 2 * bigF + 128);
    // large tables: 4x the largest estimate of any system (and never smaller than 4x the medium ones)
    s->bigCaps.CT = (int)std::max<long long>(std::max(s->midCaps.CT * 4, std::min(n, 4096)), 4 * bigT);
    s->bigCaps.CF = next_pow2_ll(std::max<long long>(4LL * s->midCaps.CF, 6 * (bigF + bigT)));
    s->bigCaps.CV = next_pow2_ll(std::max<long long>(4LL * s->midCaps.CV, 8 * bigV));
    s->bigCaps.CW = (int)std::max<long long>(4LL * s->midCaps.CW, 24 * bigF + 1024);
    s->bigCaps.CL = (int)std::max<long long>(4LL * s->midCaps.CL, 4 * bigV + 256);
    s->bigCaps.CLOG = (int)std::max<long long>(4LL * s->midCaps.CLOG + 8 * s->bigCaps.CT, 16 * bigT + 8 * bigF);
    s->maxWindows = (int)std::min<long long>(1 << 30, 200 * maxF + 20000);
    s->midMaxWindows = (int)std::min<long long>(1 << 30, 200 * bigF + 20000);
    s->bigMaxWindows = (int)std::min<long long>(1 << 30, 400 * bigF + 100000);
    s->slotBytes = cssg_geo_slot_bytes(s->caps);
    s->midSlotBytes = cssg_geo_slot_bytes(s->midCaps);
    s->bigSlotBytes = cssg_geo_slot_bytes(s->bigCaps);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    s->nSlots = std::min(n, sms * 32);
    s->nSlots = ((s->nSlots + 7) / 8) * 8;
    s->nBigSlots = std::min(n, sms);
    // medium pass: up to 16 warps per SM when some system is routed there, else a token pass for overflows; the
    // slot count is capped so that the medium scratch stays within 8 GB
    {
        long long want = anyBig ? (long long)sms * 16 : (long long)sms;
        long long fit = std::max<long long>(1, (8LL << 30) / (long long)s->midSlotBytes);
        s->nMidSlots = (int)std::max<long long>(1, std::min<long long>({(long long)n, want, fit}));
        s->midSlotsMax = s->nMidSlots;
    }
    TRY(alloc(&s->scratch, s->slotBytes * (size_t)s->nSlots));
    TRY(alloc(&s->midScratch, s->midSlotBytes * (size_t)s->nMidSlots));
    TRY(alloc(&s->bigScratch, s->bigSlotBytes * (size_t)s->nBigSlots));
    cssg_geo_init_scratch(s->scratch, s->slotBytes, s->nSlots, s->caps, ctx->stream);
    cssg_geo_init_scratch(s->midScratch, s->midSlotBytes, s->nMidSlots, s->midCaps, ctx->stream);
    cssg_geo_init_scratch(s->bigScratch, s->bigSlotBytes, s->nBigSlots, s->bigCaps, ctx->stream);
    TRY(alloc((void**)&s->chains, sizeof(double) * chain_len(s) * K));
    cudaMemset(s->chains, 0, sizeof(double) * chain_len(s) * K);
    if (s->P.integrator == 1) TRY(reset_chain(s));
    CSSG_CUDA(cudaStreamSynchronize(ctx->stream));
    CSSG_CUDA(cudaGetLastError());
#undef TRY
    *out = s;
    return CSSG_OK;
}

extern "C" int cssg_system_create(cssg_ctx* ctx, const cssg_mesh* mesh, int n, const cssg_params* params,
                                  cssg_system** out)
{
    if (!mesh || n <= 0) {
        cssg_set_error("cssg_system_create: bad arguments");
        return CSSG_ERR_ARG;
    }
    return cssg_system_create_batched(ctx, 1, &mesh, &n, params, out);
}

extern "C" int cssg_system_destroy(cssg_system* s)
{
    if (!s) return CSSG_OK;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    if (s->graphExec) cudaGraphExecDestroy(s->graphExec);
    if (s->graphAudit) cudaGraphExecDestroy(s->graphAudit);
    for (cudaEvent_t e : s->events) cudaEventDestroy(e);
    void* ptrs[] = {s->face, s->bary, s->vel, s->force, s->disp, s->pos, s->walkStatus, s->srcStatus,
                    s->statusBits, s->counters, s->cellOf, s->cellCount, s->cellStart, s->cellCursor, s->cellList,
                    s->slotOf, s->scanBlocks, s->scratch, s->midScratch, s->bigScratch, s->work, s->failList,
                    s->failList2, s->srcCost, s->lptOrder, s->lptBuckets, s->fireState, s->fireTrans,
                    s->fireDone, s->stressPartials, s->pairD, s->pairT,
                    s->pairJ, s->pairCount, s->chains, s->ke, s->dsys, s->dmeshes, s->sysOf, s->dPartBase,
                    s->mlpParams, s->candJPad, s->candCount, s->maxChord, s->candOff, s->pairI, s->pairJc, s->X,
                    s->chordS, s->yhat, s->skip, s->candScanBlocks, s->mlpErr, s->screenCounters, s->dsysScreen,
                    s->forceAudit, s->inRangeScr, s->inRangeExact, s->screenOff, s->auditCounters, s->laneScratch};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete s;
    return CSSG_OK;
}

extern "C" int cssg_system_set_state(cssg_system* s, const int* face, const double* bary, const double* vel,
                                     const double* force)
{
    if (!s) return cssg_bad_args("cssg_system_set_state");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    if (face) {
        for (int k = 0; k < s->K; ++k)
            for (int i = s->partBase[k]; i < s->partBase[k + 1]; ++i)
                if (face[i] < 0 || face[i] >= s->meshes[k]->d.nF) {
                    cssg_set_error("cssg_system_set_state: face index out of range");
                    return CSSG_ERR_ARG;
                }
        CSSG_CUDA(cudaMemcpyAsync(s->face, face, sizeof(int) * n, cudaMemcpyHostToDevice, st));
    }
    if (bary) CSSG_CUDA(cudaMemcpyAsync(s->bary, bary, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (vel) CSSG_CUDA(cudaMemcpyAsync(s->vel, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (force) CSSG_CUDA(cudaMemcpyAsync(s->force, force, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    cssg_launch_positions(s->dmeshes, s->sysOf, n, s->face, s->bary, s->pos, st);
    CSSG_CUDA(cudaStreamSynchronize(st));
    return CSSG_OK;
}

extern "C" int cssg_system_reset_thermostat(cssg_system* s)
{
    if (!s) return cssg_bad_args("cssg_system_reset_thermostat");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    return reset_chain(s);
}

extern "C" int cssg_system_kernels_per_step(cssg_system* s, int* count)
{
    if (!s || !count) return cssg_bad_args("cssg_system_kernels_per_step");
    // forces: [cell list: assign, scan x3, scatter, sort] + [screen: candidates, clamp, scan x3, compact, features,
    // inference, decisions, counts] + [longest-first order: 1 or 3] + three geodesic passes; NVE: walk (with both
    // kicks folded in) + forces; NVT: chain, scale, walk, forces, kick, KE, walk, chain, scale
    // with the lane pass: its candidate rows (no screen), the segmented order (1; the global one with a split) and,
    // with a split, the group pass over the costliest sources
    const int split = s->laneLanes > 0 && s->laneSplit > 0 ? 1 : 0;
    const int global = s->n <= kLptSmallMax ? 1 : 3;
    const int lpt = split ? global : (s->tuneLpt ? (s->laneLanes > 0 ? 1 : global) : 0);
    const int forces = (s->useCells ? 6 : 0) + (s->screen ? 10 : (s->laneLanes > 0 ? 1 : 0)) + lpt + split + 3;
    *count = s->P.integrator == 0 ? 1 + forces : 8 + forces;
    return CSSG_OK;
}

extern "C" int cssg_system_kernels_per_audit_step(cssg_system* s, int* count)
{
    if (!s || !count) return cssg_bad_args("cssg_system_kernels_per_audit_step");
    int base = 0;
    if (int rc = cssg_system_kernels_per_step(s, &base)) return rc;
    if (!(s->screen && s->auditEvery > 0)) {
        *count = base;
        return CSSG_OK;
    }
    // the exact pass on the same positions (no cell list, no screen chain; the lane pass's candidate rows) and the
    // comparison kernel
    const int split = s->laneLanes > 0 && s->laneSplit > 0 ? 1 : 0;
    const int global = s->n <= kLptSmallMax ? 1 : 3;
    const int lpt = split ? global : (s->tuneLpt ? (s->laneLanes > 0 ? 1 : global) : 0);
    *count = base + lpt + (s->laneLanes > 0 ? 1 : 0) + split + 3 + 1;
    return CSSG_OK;
}

extern "C" int cssg_system_get_state(cssg_system* s, int* face, double* bary, double* vel, double* force)
{
    if (!s) return cssg_bad_args("cssg_system_get_state");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    if (face) CSSG_CUDA(cudaMemcpyAsync(face, s->face, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    if (bary) CSSG_CUDA(cudaMemcpyAsync(bary, s->bary, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (vel) CSSG_CUDA(cudaMemcpyAsync(vel, s->vel, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (force) CSSG_CUDA(cudaMemcpyAsync(force, s->force, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaStreamSynchronize(st));
    return CSSG_OK;
}

extern "C" int cssg_system_device_state(cssg_system* s, int** face, double** bary, double** vel, double** force)
{
    if (!s) return cssg_bad_args("cssg_system_device_state");
    if (face) *face = s->face;
    if (bary) *bary = s->bary;
    if (vel) *vel = s->vel;
    if (force) *force = s->force;
    return CSSG_OK;
}

namespace {
// captures one step (the audit variant when audit is set) into a graph
int capture_step(cssg_system* s, bool audit, cudaGraphExec_t* out)
{
    cudaStream_t st = s->ctx->stream;
    cudaGraph_t g;
    s->auditStep = audit;
    CSSG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    launch_step(s);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    s->auditStep = false;
    if (e != cudaSuccess) return cssg_cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *out = nullptr;
        return cssg_cuda_fail(e, "cudaGraphInstantiate");
    }
    return CSSG_OK;
}
}  // namespace

extern "C" int cssg_system_step(cssg_system* s, int steps, int use_graph)
{
    if (!s || steps < 0) return cssg_bad_args("cssg_system_step");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    s->eventsUsed = 0;
    const bool audits = s->screen && s->auditEvery > 0;
    if (use_graph && !s->timing) {
        if (!s->graphExec)
            if (int rc = capture_step(s, false, &s->graphExec)) return rc;
        if (audits && !s->graphAudit)
            if (int rc = capture_step(s, true, &s->graphAudit)) return rc;
        for (int k = 0; k < steps; ++k) {
            const bool audit = audits && (++s->stepsDone % s->auditEvery) == 0;
            CSSG_CUDA(cudaGraphLaunch(audit ? s->graphAudit : s->graphExec, st));
        }
    } else {
        if (s->timing) {
            size_t need = (size_t)steps * 12 + 8;
            while (s->events.size() < need) {
                cudaEvent_t e;
                CSSG_CUDA(cudaEventCreate(&e));
                s->events.push_back(e);
            }
        }
        for (int k = 0; k < steps; ++k) {
            s->auditStep = audits && (++s->stepsDone % s->auditEvery) == 0;
            launch_step(s);
            s->auditStep = false;
        }
    }
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}

extern "C" int cssg_system_step_host(cssg_system* s, int steps, const int* face_in, const double* bary_in,
                                     const double* vel_in, const double* force_in, int* face_out, double* bary_out,
                                     double* vel_out, double* force_out)
{
    if (!s || steps < 0) return cssg_bad_args("cssg_system_step_host");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    if (face_in) {
        for (int k = 0; k < s->K; ++k)
            for (int i = s->partBase[k]; i < s->partBase[k + 1]; ++i)
                if (face_in[i] < 0 || face_in[i] >= s->meshes[k]->d.nF) {
                    cssg_set_error("cssg_system_step_host: face index out of range");
                    return CSSG_ERR_ARG;
                }
        CSSG_CUDA(cudaMemcpyAsync(s->face, face_in, sizeof(int) * n, cudaMemcpyHostToDevice, st));
    }
    if (bary_in) CSSG_CUDA(cudaMemcpyAsync(s->bary, bary_in, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (vel_in) CSSG_CUDA(cudaMemcpyAsync(s->vel, vel_in, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (force_in) CSSG_CUDA(cudaMemcpyAsync(s->force, force_in, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (face_in || bary_in) cssg_launch_positions(s->dmeshes, s->sysOf, n, s->face, s->bary, s->pos, st);
    const int rc = cssg_system_step(s, steps, 1);
    if (rc != CSSG_OK) return rc;
    if (face_out) CSSG_CUDA(cudaMemcpyAsync(face_out, s->face, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    if (bary_out) CSSG_CUDA(cudaMemcpyAsync(bary_out, s->bary, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (vel_out) CSSG_CUDA(cudaMemcpyAsync(vel_out, s->vel, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    if (force_out) CSSG_CUDA(cudaMemcpyAsync(force_out, s->force, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaStreamSynchronize(st));
    return CSSG_OK;
}

extern "C" int cssg_system_compute_forces(cssg_system* s)
{
    if (!s) return cssg_bad_args("cssg_system_compute_forces");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    s->eventsUsed = 0;
    launch_forces(s);
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}

namespace {
void drop_graph(cssg_system* s)
{
    if (s->graphExec) {
        cudaGraphExecDestroy(s->graphExec);
        s->graphExec = nullptr;
    }
    if (s->graphAudit) {
        cudaGraphExecDestroy(s->graphAudit);
        s->graphAudit = nullptr;
    }
}
}  // namespace

extern "C" int cssg_system_set_tuning(cssg_system* s, double delta_scale, int warps_per_block, int mid_slots,
                                      int warps_per_sm, int lpt_order, int warps_per_source, int wide_registers)
{
    if (!s || !(delta_scale > 0) || warps_per_block < 1 || warps_per_block > 8 || warps_per_sm < 0 ||
        (warps_per_source != 1 && warps_per_source != 2 && warps_per_source != 4 && warps_per_source != 8) ||
        wide_registers < 0 || wide_registers > 3) {
        cssg_set_error("cssg_system_set_tuning: bad arguments (delta_scale > 0, 1 <= warps_per_block <= 8, "
                       "warps_per_sm >= 0, warps_per_source in {1, 2, 4, 8}, kernel build 0..3)");
        return CSSG_ERR_ARG;
    }
    s->tuneGroup = warps_per_source;
    s->tuneWide = wide_registers;
    s->tuneDelta = delta_scale;
    s->tuneWpb = warps_per_block;
    if (mid_slots > 0) s->nMidSlots = std::min(mid_slots, s->midSlotsMax);
    s->tuneWarpsPerSM = warps_per_sm;
    s->tuneLpt = lpt_order != 0;
    drop_graph(s);
    return CSSG_OK;
}

// Times compute_forces (the propagation passes) on the current state for each candidate (band width scale x warps
// per block x medium slots) and keeps the fastest.  Forces are recomputed on the same state, so the physics does
// not change; the result differs between candidates only in the work done.
extern "C" int cssg_system_autotune(cssg_system* s, int reps, double* result_host)
{
    if (!s) return cssg_bad_args("cssg_system_autotune");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    if (reps < 1) reps = 1;
    cudaStream_t st = s->ctx->stream;
    int sms = 0;
    CSSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->ctx->device));
    const double deltas[] = {0.5, 1.0, 2.0, 4.0};
    // (warps per block, warps per SM cap, longest-first order, warps per source, wide registers)
    const int shapes[][5] = {{8, 0, 0, 1, 0}, {4, 0, 0, 1, 0}, {8, 0, 1, 1, 0}, {8, 8, 1, 1, 0}, {8, 4, 1, 1, 0},
                             {8, 0, 1, 2, 0}, {8, 0, 1, 4, 0}, {8, 0, 1, 8, 0}, {8, 0, 1, 1, 1}, {8, 0, 1, 2, 1},
                             {8, 0, 1, 4, 1}, {8, 0, 1, 1, 3}, {8, 0, 1, 1, 2}, {8, 0, 1, 2, 3}};
    std::vector<int> mids{s->midSlotsMax};
    if (s->midSlotsMax > sms * 8) mids.push_back(sms * 8);
    cudaEvent_t e0, e1;
    CSSG_CUDA(cudaEventCreate(&e0));
    CSSG_CUDA(cudaEventCreate(&e1));
    double best = 1e300, bd = s->tuneDelta;
    int bw = s->tuneWpb, bm = s->nMidSlots, bc = s->tuneWarpsPerSM, bg = s->tuneGroup, bx = s->tuneWide;
    bool bl = s->tuneLpt;
    const bool timing = s->timing;
    s->timing = false;
    // status bits raised before the call are kept; a candidate that raises any (a capacity overflow) is rejected
    int prior = 0;
    CSSG_CUDA(cudaMemcpyAsync(&prior, s->statusBits, sizeof(int), cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaStreamSynchronize(st));
    s->laneLanes = 0;  // the source-group candidates first, every pass with the same group size
    s->tuneMidGroup = s->tuneBigGroup = 0;
    for (double d : deltas)
        for (const auto& sh : shapes)
            for (int m : mids) {
                s->tuneDelta = d;
                s->tuneWpb = sh[0];
                s->tuneWarpsPerSM = sh[1];
                s->tuneLpt = sh[2] != 0;
                s->tuneGroup = sh[3];
                s->tuneWide = sh[4];
                s->nMidSlots = m;
                launch_forces(s);  // warm-up of this configuration
                cudaEventRecord(e0, st);
                for (int r = 0; r < reps; ++r) launch_forces(s);
                cudaEventRecord(e1, st);
                cudaError_t err = cudaEventSynchronize(e1);
                if (err != cudaSuccess) {
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    return cssg_cuda_fail(err, "cssg_system_autotune");
                }
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                int bits = 0;
                cudaMemcpy(&bits, s->statusBits, sizeof(int), cudaMemcpyDeviceToHost);
                cudaMemset(s->statusBits, 0, sizeof(int));
                if (bits == 0 && ms < best) {
                    best = ms;
                    bd = d;
                    bw = sh[0];
                    bc = sh[1];
                    bl = sh[2] != 0;
                    bg = sh[3];
                    bx = sh[4];
                    bm = m;
                }
            }
    // the one-source-per-lane pass (16 or 32 sources per warp, cell or longest-first order); the group tuning found
    // above still serves the sources it hands to the medium and large passes
    int bLanes = 0, bSplit = 0;
    const bool blGroup = bl;  // the source groups' order choice, kept if the lane pass is not taken
    // single-system objects only: on the 64-system batch the lane pass with a split timed 28 ms per evaluation here
    // but 47 ms in the steps that followed (uneven systems whose costs move), while source groups held 32 ms
    if (s->useCells && s->K == 1) {
        s->tuneDelta = bd;
        s->tuneWpb = bw;
        s->tuneWarpsPerSM = bc;
        s->tuneGroup = bg;
        s->tuneWide = bx;
        s->nMidSlots = bm;
        // splits: none, or the costliest 1/64, 1/16 or 1/4 of the sources to the group pass
        const int splits[] = {0, s->n / 64, s->n / 16, s->n / 4};
        for (int lanes : {16, 32})
            for (int lpt = 0; lpt < 2; ++lpt)
                for (int sp = 0; sp < 4; ++sp) {
                    if (sp > 0 && (lpt == 0 || splits[sp] == 0)) continue;  // a split always orders by cost
                    if (set_lanes(s, lanes) != CSSG_OK) break;
                    s->laneSplit = splits[sp];
                    s->tuneLpt = lpt != 0;
                    launch_forces(s);
                    launch_forces(s);  // warm-up (and the longest-first order from a lane-pass evaluation)
                    cudaEventRecord(e0, st);
                    for (int r = 0; r < reps; ++r) launch_forces(s);
                    cudaEventRecord(e1, st);
                    cudaError_t err = cudaEventSynchronize(e1);
                    if (err != cudaSuccess) {
                        cudaEventDestroy(e0);
                        cudaEventDestroy(e1);
                        return cssg_cuda_fail(err, "cssg_system_autotune");
                    }
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    int bits = 0;
                    cudaMemcpy(&bits, s->statusBits, sizeof(int), cudaMemcpyDeviceToHost);
                    cudaMemset(s->statusBits, 0, sizeof(int));
                    // the lane pass must beat the source groups by 5%: its time depends more on the state (a warp
                    // waits for its slowest source; the split follows the last evaluation's costs)
                    if (bits == 0 && ms < (bLanes ? best : 0.95 * best)) {
                        best = ms;
                        bLanes = lanes;
                        bSplit = splits[sp];
                        bl = lpt != 0;
                    }
                }
        if (bLanes > 0) {
            // confirm the lane pass on a steadier state (its time depends more on the state: the split follows the
            // last evaluation's costs, a warp waits for its slowest source): more evaluations of each, then the same
            // 5% margin against the best source-group configuration
            auto steady = [&](int warm, float* ms) -> cudaError_t {
                for (int r = 0; r < warm; ++r) launch_forces(s);
                cudaEventRecord(e0, st);
                for (int r = 0; r < reps; ++r) launch_forces(s);
                cudaEventRecord(e1, st);
                cudaError_t err = cudaEventSynchronize(e1);
                if (err == cudaSuccess) err = cudaEventElapsedTime(ms, e0, e1);
                int bits = 0;
                cudaMemcpy(&bits, s->statusBits, sizeof(int), cudaMemcpyDeviceToHost);
                cudaMemset(s->statusBits, 0, sizeof(int));
                if (bits) *ms = 1e30f;
                return err;
            };
            float lms = 0, gms = 0;
            set_lanes(s, bLanes);
            s->laneSplit = bSplit;
            s->tuneLpt = bl;
            cudaError_t err = steady(4, &lms);
            s->laneLanes = 0;
            s->laneSplit = 0;
            s->tuneLpt = blGroup;
            if (err == cudaSuccess) err = steady(4, &gms);
            if (err != cudaSuccess) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return cssg_cuda_fail(err, "cssg_system_autotune");
            }
            if (lms < 0.95f * gms) {
                best = lms;
            } else {
                best = gms;
                bLanes = 0;
                bSplit = 0;
                bl = blGroup;
            }
        }
        set_lanes(s, bLanes);
        s->laneSplit = bSplit;
        s->tuneLpt = bl;
    }
    // the medium and large passes take the largest sources: try 8-warp groups there (a few huge patches are the
    // tail of a force pass)
    s->tuneDelta = bd;
    s->tuneWpb = bw;
    s->tuneWarpsPerSM = bc;
    s->tuneLpt = bl;
    s->tuneGroup = bg;
    s->tuneWide = bx;
    s->nMidSlots = bm;
    int bMid = 0, bBig = 0;
    {
        // (regular, medium, large) warps per source; smaller regular groups pay off once the large sources have
        // their own 8-warp groups
        const int passGroups[][3] = {{bg, 0, 0}, {bg, 8, 0}, {bg, 8, 8}, {2, 8, 8}, {1, 8, 8}};
        bool first = true;
        for (int c = 0; c < 5; ++c) {
            const int* pg = passGroups[c];
            if ((c == 1 || c == 2) && bg == 8) continue;  // 8-warp passes are the regular pass's own groups
            if (c >= 3 && pg[0] >= bg) continue;          // only smaller regular groups than the chosen one
            s->tuneGroup = pg[0];
            s->tuneMidGroup = pg[1];
            s->tuneBigGroup = pg[2];
            launch_forces(s);
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps; ++r) launch_forces(s);
            cudaEventRecord(e1, st);
            cudaError_t err = cudaEventSynchronize(e1);
            if (err != cudaSuccess) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return cssg_cuda_fail(err, "cssg_system_autotune");
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            int bits = 0;
            cudaMemcpy(&bits, s->statusBits, sizeof(int), cudaMemcpyDeviceToHost);
            cudaMemset(s->statusBits, 0, sizeof(int));
            // the first candidate re-times the configuration chosen above (the reference for the others)
            if (bits == 0 && (first || ms < best)) {
                best = ms;
                bg = pg[0];
                bMid = pg[1];
                bBig = pg[2];
            }
            first = false;
        }
    }
    s->tuneMidGroup = bMid;
    s->tuneBigGroup = bBig;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->timing = timing;
    s->tuneDelta = bd;
    s->tuneWpb = bw;
    s->tuneWarpsPerSM = bc;
    s->tuneLpt = bl;
    s->tuneGroup = bg;
    s->tuneWide = bx;
    s->nMidSlots = bm;
    drop_graph(s);
    // leave the forces of the current state computed with the chosen configuration
    launch_forces(s);
    CSSG_CUDA(cudaStreamSynchronize(st));
    if (prior) {
        int bits = 0;
        CSSG_CUDA(cudaMemcpy(&bits, s->statusBits, sizeof(int), cudaMemcpyDeviceToHost));
        bits |= prior;
        CSSG_CUDA(cudaMemcpy(s->statusBits, &bits, sizeof(int), cudaMemcpyHostToDevice));
    }
    CSSG_CUDA(cudaGetLastError());
    if (result_host) {
        result_host[0] = bd;
        result_host[1] = bw;
        result_host[2] = bm;
        result_host[3] = bc;
        result_host[4] = bl ? 1 : 0;
        result_host[5] = best / reps;
        result_host[6] = bg;
        result_host[7] = bx;
    }
    return CSSG_OK;
}

extern "C" int cssg_system_check(cssg_system* s, int* bits, unsigned long long* counters)
{
    if (!s) return cssg_bad_args("cssg_system_check");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    int hb = 0;
    unsigned long long hc[8];
    CSSG_CUDA(cudaMemcpyAsync(&hb, s->statusBits, sizeof(int), cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaMemcpyAsync(hc, s->counters, sizeof(hc), cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaMemsetAsync(s->statusBits, 0, sizeof(int), st));
    CSSG_CUDA(cudaMemsetAsync(s->counters, 0, sizeof(hc), st));
    CSSG_CUDA(cudaStreamSynchronize(st));
    if (bits) *bits = hb;
    if (counters)
        for (int k = 0; k < 5; ++k) counters[k] = hc[k];
    return CSSG_OK;
}

extern "C" int cssg_system_pairs(cssg_system* s, int cap, int* ih, int* jh, double* dh, double* th, int* count)
{
    if (!s) return cssg_bad_args("cssg_system_pairs");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    if (!s->pairD) {
        // enable pair output for subsequent force evaluations
        s->pairCap = std::max(16, s->caps.CT);
        size_t slots = (size_t)s->n * s->pairCap;
        int rc;
        if ((rc = alloc((void**)&s->pairD, sizeof(double) * slots)) || (rc = alloc((void**)&s->pairT, sizeof(double) * 3 * slots)) ||
            (rc = alloc((void**)&s->pairJ, sizeof(int) * slots)) || (rc = alloc((void**)&s->pairCount, sizeof(int) * s->n)))
            return rc;
        drop_graph(s);
        CSSG_CUDA(cudaMemsetAsync(s->pairCount, 0, sizeof(int) * s->n, st));
        if (count) *count = 0;
        CSSG_CUDA(cudaStreamSynchronize(st));
        return CSSG_OK;
    }
    std::vector<int> cnt(s->n);
    size_t slots = (size_t)s->n * s->pairCap;
    std::vector<double> d(slots), t(3 * slots);
    std::vector<int> j(slots);
    CSSG_CUDA(cudaMemcpyAsync(cnt.data(), s->pairCount, sizeof(int) * s->n, cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaMemcpyAsync(d.data(), s->pairD, sizeof(double) * slots, cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaMemcpyAsync(t.data(), s->pairT, sizeof(double) * 3 * slots, cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaMemcpyAsync(j.data(), s->pairJ, sizeof(int) * slots, cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaStreamSynchronize(st));
    int total = 0;
    for (int i = 0; i < s->n; ++i)
        for (int q = 0; q < cnt[i] && q < s->pairCap; ++q) {
            if (total < cap) {
                size_t o = (size_t)i * s->pairCap + q;
                if (ih) ih[total] = i;
                if (jh) jh[total] = j[o];
                if (dh) dh[total] = d[o];
                if (th)
                    for (int c = 0; c < 3; ++c) th[3 * total + c] = t[3 * o + c];
            }
            total++;
        }
    if (count) *count = total;
    return CSSG_OK;
}

extern "C" int cssg_system_chain(cssg_system* s, double* chain, int capacity)
{
    if (!s || !chain) return cssg_bad_args("cssg_system_chain");
    int len = chain_len(s) * s->K;
    if (capacity < len) {
        cssg_set_error("cssg_system_chain: capacity too small");
        return CSSG_ERR_CAPACITY;
    }
    CSSG_CUDA(cudaMemcpyAsync(chain, s->chains, sizeof(double) * len, cudaMemcpyDeviceToHost, s->ctx->stream));
    CSSG_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return CSSG_OK;
}

// Learned screen on/off.  params_host: cssg_mlp_param_count() FP32 values (nullable when disabling); a pair is
// skipped when |chord| / sigma + yhat > 1 + margin.  Requires the cell-list neighbour structure.
extern "C" int cssg_system_set_screen(cssg_system* s, const float* params_host, double margin, int enable)
{
    if (!s) return cssg_bad_args("cssg_system_set_screen");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    if (enable) {
        if (!s->useCells || !params_host) {
            cssg_set_error("cssg_system_set_screen: needs parameters and the cell-list neighbour structure");
            return CSSG_ERR_ARG;
        }
        const int n = s->n;
        if (!s->mlpParams) {
            if (int rc = ensure_candidate_rows(s)) return rc;
            size_t slots = (size_t)n * s->candCap;
            int rc;
            s->nCandScanBlocks = (n + SCAN_BLOCK * SCAN_ITEMS - 1) / (SCAN_BLOCK * SCAN_ITEMS);
            if ((rc = alloc((void**)&s->mlpParams, sizeof(float) * cssg_mlp_param_count())) ||
                (rc = alloc((void**)&s->candOff, sizeof(int) * (n + 1))) ||
                (rc = alloc((void**)&s->pairI, sizeof(int) * slots)) ||
                (rc = alloc((void**)&s->pairJc, sizeof(int) * slots)) ||
                (rc = alloc(&s->X, 32 * slots)) || (rc = alloc((void**)&s->chordS, sizeof(float) * slots)) ||
                (rc = alloc((void**)&s->yhat, sizeof(float) * slots)) ||
                (rc = alloc((void**)&s->skip, slots)) ||
                (rc = alloc((void**)&s->candScanBlocks, sizeof(int) * (s->nCandScanBlocks + 1))) ||
                (rc = alloc((void**)&s->mlpErr, sizeof(int))) ||
                (rc = alloc((void**)&s->screenCounters, sizeof(unsigned long long) * 2)) ||
                (rc = alloc((void**)&s->dsysScreen, sizeof(SysDesc) * s->K)) ||
                (rc = alloc((void**)&s->forceAudit, sizeof(double) * 3 * n)) ||
                (rc = alloc((void**)&s->inRangeScr, sizeof(int) * n)) ||
                (rc = alloc((void**)&s->inRangeExact, sizeof(int) * n)) ||
                (rc = alloc((void**)&s->screenOff, sizeof(int))) ||
                (rc = alloc((void**)&s->auditCounters, sizeof(unsigned long long) * 2)))
                return rc;
            CSSG_CUDA(cudaMemset(s->auditCounters, 0, sizeof(unsigned long long) * 2));
            std::vector<SysDesc> h = s->hsys;
            for (auto& d : h) d.searchMode = 3;
            CSSG_CUDA(cudaMemcpy(s->dsysScreen, h.data(), sizeof(SysDesc) * s->K, cudaMemcpyHostToDevice));
            CSSG_CUDA(cudaMemset(s->mlpErr, 0, sizeof(int)));
            CSSG_CUDA(cudaMemset(s->screenCounters, 0, sizeof(unsigned long long) * 2));
        }
        CSSG_CUDA(cudaMemcpyAsync(s->mlpParams, params_host, sizeof(float) * cssg_mlp_param_count(),
                                  cudaMemcpyHostToDevice, st));
        CSSG_CUDA(cudaMemsetAsync(s->screenOff, 0, sizeof(int), st));  // (re-)enabling clears an audit's fallback
        CSSG_CUDA(cudaStreamSynchronize(st));
        s->margin = margin;
    }
    s->screen = enable != 0;
    drop_graph(s);
    return CSSG_OK;
}

// {candidate pairs, screened-out pairs, tensor-core wait failures} since the last call (synchronises, resets)
extern "C" int cssg_system_screen_counters(cssg_system* s, unsigned long long* out_host)
{
    if (!s || !out_host) return cssg_bad_args("cssg_system_screen_counters");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    out_host[0] = out_host[1] = out_host[2] = 0;
    if (!s->screenCounters) return CSSG_OK;
    cudaStream_t st = s->ctx->stream;
    unsigned long long h[2];
    int e = 0;
    CSSG_CUDA(cudaMemcpyAsync(h, s->screenCounters, sizeof(h), cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaMemcpyAsync(&e, s->mlpErr, sizeof(int), cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaMemsetAsync(s->screenCounters, 0, sizeof(h), st));
    CSSG_CUDA(cudaMemsetAsync(s->mlpErr, 0, sizeof(int), st));
    CSSG_CUDA(cudaStreamSynchronize(st));
    out_host[0] = h[0];
    out_host[1] = h[1];
    out_host[2] = (unsigned long long)e;
    return CSSG_OK;
}

extern "C" int cssg_system_set_lanes(cssg_system* s, int lanes_per_warp)
{
    if (!s || (lanes_per_warp != 0 && lanes_per_warp != 16 && lanes_per_warp != 32))
        return cssg_bad_args("cssg_system_set_lanes");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    if (int rc = set_lanes(s, lanes_per_warp)) return rc;
    drop_graph(s);
    return CSSG_OK;
}

extern "C" int cssg_system_lanes(cssg_system* s, int* lanes_per_warp)
{
    if (!s || !lanes_per_warp) return cssg_bad_args("cssg_system_lanes");
    *lanes_per_warp = s->laneLanes;
    return CSSG_OK;
}

extern "C" int cssg_system_set_lane_split(cssg_system* s, int group_sources)
{
    if (!s || group_sources < 0) return cssg_bad_args("cssg_system_set_lane_split");
    s->laneSplit = std::min(group_sources, s->n);
    drop_graph(s);
    return CSSG_OK;
}

extern "C" int cssg_system_lane_split(cssg_system* s, int* group_sources)
{
    if (!s || !group_sources) return cssg_bad_args("cssg_system_lane_split");
    *group_sources = s->laneSplit;
    return CSSG_OK;
}

extern "C" int cssg_system_set_pass_groups(cssg_system* s, int medium_warps, int large_warps)
{
    auto ok = [](int g) { return g == 0 || g == 1 || g == 2 || g == 4 || g == 8; };
    if (!s || !ok(medium_warps) || !ok(large_warps)) return cssg_bad_args("cssg_system_set_pass_groups");
    s->tuneMidGroup = medium_warps;
    s->tuneBigGroup = large_warps;
    drop_graph(s);
    return CSSG_OK;
}

extern "C" int cssg_system_pass_groups(cssg_system* s, int* medium_warps, int* large_warps)
{
    if (!s || !medium_warps || !large_warps) return cssg_bad_args("cssg_system_pass_groups");
    *medium_warps = s->tuneMidGroup;
    *large_warps = s->tuneBigGroup;
    return CSSG_OK;
}

extern "C" int cssg_system_source_costs(cssg_system* s, int capacity, int* cost_host)
{
    if (!s || !cost_host || capacity < s->n) return cssg_bad_args("cssg_system_source_costs");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    CSSG_CUDA(cudaMemcpyAsync(cost_host, s->srcCost, sizeof(int) * s->n, cudaMemcpyDeviceToHost, s->ctx->stream));
    CSSG_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return CSSG_OK;
}

extern "C" int cssg_system_set_work_caps(cssg_system* s, int regular, int medium, int large)
{
    if (!s) return cssg_bad_args("cssg_system_set_work_caps");
    if (regular > 0) s->maxWindows = regular;
    if (medium > 0) s->midMaxWindows = medium;
    if (large > 0) s->bigMaxWindows = large;
    drop_graph(s);
    return CSSG_OK;
}

extern "C" int cssg_system_set_screen_audit(cssg_system* s, int every)
{
    if (!s || every < 0) return cssg_bad_args("cssg_system_set_screen_audit");
    s->auditEvery = every;
    s->stepsDone = 0;
    drop_graph(s);
    return CSSG_OK;
}

extern "C" int cssg_system_screen_audit_status(cssg_system* s, long long* out_host)
{
    if (!s || !out_host) return cssg_bad_args("cssg_system_screen_audit_status");
    out_host[0] = out_host[1] = out_host[2] = 0;
    if (!s->auditCounters) return CSSG_OK;
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    unsigned long long h[2];
    int off = 0;
    CSSG_CUDA(cudaMemcpyAsync(h, s->auditCounters, sizeof(h), cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaMemcpyAsync(&off, s->screenOff, sizeof(int), cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaStreamSynchronize(st));
    out_host[0] = (long long)h[0];
    out_host[1] = (long long)h[1];
    out_host[2] = off;
    return CSSG_OK;
}

extern "C" int cssg_system_timing(cssg_system* s, int enable)
{
    if (!s) return cssg_bad_args("cssg_system_timing");
    s->timing = enable != 0;
    return CSSG_OK;
}

// ms[0] = geodesic/force kernel total, ms[1] = walk kernel total over the last step() call
extern "C" int cssg_system_last_times(cssg_system* s, double* ms, int capacity)
{
    if (!s || !ms || capacity < 2) return cssg_bad_args("cssg_system_last_times");
    CSSG_CUDA(cudaStreamSynchronize(s->ctx->stream));
    double geo = 0, walk = 0;
    // events are recorded in pairs: (geo start, geo end) and (walk start, walk end) in launch order
    // a launch_forces call records 2 events, a launch_walk call records 2 events
    // the order is deterministic per integrator: NVE: walk, forces ; NVT: walk, forces, walk
    int perStep = s->P.integrator == 0 ? 4 : 6;
    int steps = s->eventsUsed / perStep;
    for (int k = 0; k < steps; ++k) {
        int b = k * perStep;
        float ms0 = 0;
        // walk first
        cudaEventElapsedTime(&ms0, s->events[b], s->events[b + 1]);
        walk += ms0;
        cudaEventElapsedTime(&ms0, s->events[b + 2], s->events[b + 3]);
        geo += ms0;
        if (perStep == 6) {
            cudaEventElapsedTime(&ms0, s->events[b + 4], s->events[b + 5]);
            walk += ms0;
        }
    }
    ms[0] = geo;
    ms[1] = walk;
    return CSSG_OK;
}


// ---------------------------------------------------------------------------------------------------------------------
// FIRE minimisation: fireMinimization::minimizeByFire (src/updaters/fireMinimization.cpp:3-21) on the device.  One
// iteration = velocity-Verlet half step, walk with force and velocity transported (simpleModel::moveParticles with both
// transport flags, force first), forces, second half step, fireStep (:38-77), getMaxForce (baseUpdater.cpp:39-54).
// The scalar state (deltaT, alpha, nSinceNegativePower, iteration count, stop flag) lives on the device, so a chunk of
// iterations is one graph replay; every kernel that changes state returns at once when the stop flag is set, and the
// host reads the flag once per chunk.
// ---------------------------------------------------------------------------------------------------------------------
namespace {

struct FireState {
    double dt, alpha, mixAlpha, mixScale, forceMax;
    double alphaStart, dtMax, dtMin, dtInc, dtDec, alphaDec, forceCutoff, alphaMin;
    int nMin, maxIterations, nSince, iterations, done, resetV;
};

constexpr int kFireBlock = 256;
constexpr int kFireChunk = 16;

// Each system of a batched object has its own FireState (deltaT, alpha, counters, stop flag) and stops on its own:
// the per-particle kernels leave the particles of a stopped system alone, and the walk skips them (fireDone[k]).
__device__ __forceinline__ const FireState& fire_of(const FireState* st, const int* sysOf, int i)
{
    return st[sysOf ? sysOf[i] : 0];
}

__global__ void fire_first_half(int n, const int* __restrict__ sysOf, double* __restrict__ v,
                                const double* __restrict__ f, double* __restrict__ disp, double* __restrict__ trans,
                                const FireState* __restrict__ st)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const FireState& S = fire_of(st, sysOf, i);
    if (S.done) return;
    const double dt = S.dt;
    for (int c = 0; c < 3; ++c) {
        const int k = 3 * i + c;
        disp[k] = dt * v[k] + 0.5 * dt * dt * f[k];
        v[k] += 0.5 * dt * f[k];
        trans[6 * i + c] = f[k];
        trans[6 * i + 3 + c] = v[k];
    }
}

// the transported velocity back, then (after the forces) the second half kick v += dt/2 f
__global__ void fire_unpack(int n, const int* __restrict__ sysOf, const double* __restrict__ trans,
                            double* __restrict__ v, const FireState* st)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fire_of(st, sysOf, i).done) return;
    for (int c = 0; c < 3; ++c) v[3 * i + c] = trans[6 * i + 3 + c];
}

__global__ void fire_second_half(int n, const int* __restrict__ sysOf, double* __restrict__ v,
                                 const double* __restrict__ f, const FireState* st)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const FireState& S = fire_of(st, sysOf, i);
    if (S.done) return;
    for (int c = 0; c < 3; ++c) v[3 * i + c] += 0.5 * S.dt * f[3 * i + c];
}

// fixed-order block sum of three values (every thread gets the totals)
__device__ void fire_block_sum3(double& a, double& b, double& c)
{
    __shared__ double sh[3][kFireBlock];
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = b;
    sh[2][threadIdx.x] = c;
    __syncthreads();
    for (int w = kFireBlock / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    a = sh[0][0];
    b = sh[1][0];
    c = sh[2][0];
}

// fireStep (fireMinimization.cpp:38-77) for system blockIdx.x: F.F, v.v, F.v over its particles (fixed order), the
// mixing scale, then the deltaT / alpha update on the sign of the power
__global__ void __launch_bounds__(kFireBlock) fire_scalar(const int* __restrict__ partBase,
                                                          const double* __restrict__ v, const double* __restrict__ f,
                                                          FireState* st)
{
    FireState& S = st[blockIdx.x];
    if (S.done) return;  // uniform over the block
    double forceNorm = 0, velocityNorm = 0, power = 0;
    for (int i = partBase[blockIdx.x] + threadIdx.x; i < partBase[blockIdx.x + 1]; i += kFireBlock) {
        const double* a = &f[3 * i];
        const double* b = &v[3 * i];
        forceNorm += a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        velocityNorm += b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
        power += a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    }
    fire_block_sum3(forceNorm, velocityNorm, power);
    if (threadIdx.x != 0) return;
    double scaling = 0.0;
    if (forceNorm > 0) scaling = sqrt(velocityNorm / forceNorm);
    S.mixAlpha = S.alpha;
    S.mixScale = scaling;
    if (power > 0) {
        if (S.nSince > S.nMin) {
            S.dt = fmin(S.dt * S.dtInc, S.dtMax);
            S.alpha = fmax(S.alpha * S.alphaDec, S.alphaMin);
        }
        S.nSince += 1;
        S.resetV = 0;
    } else {
        S.nSince = 0;
        S.dt = fmax(S.dt * S.dtDec, S.dtMin);
        S.alpha = S.alphaStart;
        S.resetV = 1;
    }
}

// v = (1 - alpha) v + alpha * scaling * F (zero after a non-positive power)
__global__ void fire_mix(int n, const int* __restrict__ sysOf, double* __restrict__ v, const double* __restrict__ f,
                         const FireState* st)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const FireState& S = fire_of(st, sysOf, i);
    if (S.done) return;
    const double a = S.mixAlpha, as = S.mixAlpha * S.mixScale;
    const bool reset = S.resetV != 0;
    for (int c = 0; c < 3; ++c) {
        const int k = 3 * i + c;
        v[k] = reset ? 0.0 : (1 - a) * v[k] + as * f[k];
    }
}

// getMaxForce (baseUpdater.cpp:39-54) for system blockIdx.x and the loop condition of minimizeByFire
// (fireMinimization.cpp:12-20); count = 1 after an iteration (iterations += 1), 0 for the check before the loop.
// done[k] mirrors the system's stop flag for the walk.
__global__ void __launch_bounds__(kFireBlock) fire_check(const int* __restrict__ partBase,
                                                         const double* __restrict__ f, FireState* st,
                                                         int* __restrict__ done, int count)
{
    FireState& S = st[blockIdx.x];
    if (count && S.done) return;  // uniform over the block
    double q = 0;
    for (int i = partBase[blockIdx.x] + threadIdx.x; i < partBase[blockIdx.x + 1]; i += kFireBlock)
        q = fmax(q, f[3 * i] * f[3 * i] + f[3 * i + 1] * f[3 * i + 1] + f[3 * i + 2] * f[3 * i + 2]);
    for (int o = 16; o > 0; o >>= 1) q = fmax(q, __shfl_xor_sync(0xffffffffu, q, o));
    __shared__ double sh[kFireBlock / 32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = q;
    __syncthreads();
    if (threadIdx.x != 0) return;
    double m = 0;
    for (int w = 0; w < kFireBlock / 32; ++w) m = fmax(m, sh[w]);
    S.forceMax = sqrt(m);
    if (count) S.iterations += 1;
    if (!(S.iterations < S.maxIterations && S.forceMax > S.forceCutoff)) S.done = 1;
    done[blockIdx.x] = S.done;
}

// done[K] = every system has stopped (the walk then returns at once, and the host ends the loop)
__global__ void fire_all_done(int K, int* done)
{
    if (threadIdx.x != 0) return;
    int all = 1;
    for (int k = 0; k < K; ++k) all &= done[k] != 0;
    done[K] = all;
}

void fire_iteration(cssg_system* s, FireState* dst, int nBlocks)
{
    cudaStream_t st = s->ctx->stream;
    const int n = s->n, K = s->K;
    fire_first_half<<<nBlocks, kFireBlock, 0, st>>>(n, s->sysOf, s->vel, s->force, s->disp, s->fireTrans, dst);
    cssg_launch_transport(s->dmeshes, s->sysOf, n, s->face, s->bary, s->disp, s->fireTrans, 2, s->walkStatus,
                          s->counters, s->pos, st, s->fireDone + K, s->statusBits, nullptr, 0.0, s->fireDone);
    fire_unpack<<<nBlocks, kFireBlock, 0, st>>>(n, s->sysOf, s->fireTrans, s->vel, dst);
    launch_forces(s);
    fire_second_half<<<nBlocks, kFireBlock, 0, st>>>(n, s->sysOf, s->vel, s->force, dst);
    fire_scalar<<<K, kFireBlock, 0, st>>>(s->dPartBase, s->vel, s->force, dst);
    fire_mix<<<nBlocks, kFireBlock, 0, st>>>(n, s->sysOf, s->vel, s->force, dst);
    fire_check<<<K, kFireBlock, 0, st>>>(s->dPartBase, s->force, dst, s->fireDone, 1);
    fire_all_done<<<1, 32, 0, st>>>(K, s->fireDone);
}

// stress partials per block: f(t, d) (x) t over every stored pair and, once per pair, v_i (x) v_i
__global__ void __launch_bounds__(256) stress_partials(int n, int pairCap, const int* __restrict__ pairCount,
                                                       const double* __restrict__ pairD,
                                                       const double* __restrict__ pairT,
                                                       const double* __restrict__ vel, const SysDesc* __restrict__ sys,
                                                       double* __restrict__ partials, int* __restrict__ overflow)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[18];
    for (int k = 0; k < 18; ++k) acc[k] = 0;
    if (i < n) {
        const SysDesc& D = sys[0];
        int cnt = pairCount[i];
        if (cnt > pairCap) {
            atomicExch(overflow, 1);
            cnt = pairCap;
        }
        const double v[3] = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
        for (int t = 0; t < cnt; ++t) {
            const size_t o = (size_t)i * pairCap + t;
            const double d = pairD[o];
            const double ts[3] = {pairT[3 * o], pairT[3 * o + 1], pairT[3 * o + 2]};
            double f3[3] = {0, 0, 0};
            if (d < CUDART_INF) {
                double fm = 0;
                bool use = true;
                if (D.forceKind == 0) {
                    use = d <= D.sigma;
                    if (use) fm = -D.k * (D.sigma - d);
                } else {
                    const double sqrtTwoPi = 2.50662827463100050241576528481104525300698674061;
                    fm = -(d * D.k * exp(-d * d / (2.0 * D.sigma * D.sigma)) / ((sqrtTwoPi * D.sigma) * sqrt(D.sigma)));
                }
                if (use)
                    for (int c = 0; c < 3; ++c) f3[c] = fm * ts[c];
            }
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    acc[3 * a + b] += f3[a] * ts[b];
                    acc[9 + 3 * a + b] += v[a] * v[b];
                }
        }
    }
    __shared__ double sh[18][256];
    for (int k = 0; k < 18; ++k) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 18; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 18) partials[18 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

}  // namespace

extern "C" int cssg_system_fire(cssg_system* s, const cssg_fire_params* fp, int reset, double* result_host)
{
    if (!s || !fp || fp->maximum_iterations < 0) {
        cssg_set_error("cssg_system_fire: bad arguments (maximum_iterations >= 0)");
        return CSSG_ERR_ARG;
    }
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    const int n = s->n, K = s->K;
    const int nBlocks = (n + kFireBlock - 1) / kFireBlock;
    if (!s->fireState) {
        if (int rc = alloc(&s->fireState, sizeof(FireState) * (size_t)K)) return rc;
        if (int rc = alloc((void**)&s->fireTrans, sizeof(double) * 6 * (size_t)n)) return rc;
        if (int rc = alloc((void**)&s->fireDone, sizeof(int) * (size_t)(K + 1))) return rc;
        reset = 1;
    }
    std::vector<FireState> h(K);
    FireState* dst = (FireState*)s->fireState;
    if (reset) {
        memset(h.data(), 0, sizeof(FireState) * K);
        for (auto& x : h) {
            x.dt = s->P.dt;
            x.alpha = fp->alpha_start;
        }
    } else {
        CSSG_CUDA(cudaMemcpyAsync(h.data(), dst, sizeof(FireState) * K, cudaMemcpyDeviceToHost, st));
        CSSG_CUDA(cudaStreamSynchronize(st));
    }
    for (auto& x : h) {
        x.alphaStart = fp->alpha_start;
        x.dtMax = fp->dt_max;
        x.dtMin = fp->dt_min;
        x.dtInc = fp->dt_inc;
        x.dtDec = fp->dt_dec;
        x.alphaDec = fp->alpha_dec;
        x.forceCutoff = fp->force_cutoff;
        x.alphaMin = fp->alpha_min;
        x.nMin = fp->n_min;
        x.maxIterations = fp->maximum_iterations;
        x.iterations = 0;
        x.done = 0;
    }
    CSSG_CUDA(cudaMemcpyAsync(dst, h.data(), sizeof(FireState) * K, cudaMemcpyHostToDevice, st));
    // minimizeByFire: forces and forceMax before the loop
    launch_forces(s);
    fire_check<<<K, kFireBlock, 0, st>>>(s->dPartBase, s->force, dst, s->fireDone, 0);
    fire_all_done<<<1, 32, 0, st>>>(K, s->fireDone);
    // chunks of iterations as one graph; the all-stopped flag is read after each chunk
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CSSG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < kFireChunk; ++k) fire_iteration(s, dst, nBlocks);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return cssg_cuda_fail(e, "cssg_system_fire: graph capture");
    const int maxChunks = fp->maximum_iterations / kFireChunk + 2;
    int done = 0;
    for (int c = 0; c < maxChunks; ++c) {
        CSSG_CUDA(cudaMemcpyAsync(&done, s->fireDone + K, sizeof(int), cudaMemcpyDeviceToHost, st));
        CSSG_CUDA(cudaStreamSynchronize(st));
        if (done) break;
        e = cudaGraphLaunch(ge, st);
        if (e != cudaSuccess) {
            cudaGraphExecDestroy(ge);
            return cssg_cuda_fail(e, "cssg_system_fire: graph launch");
        }
    }
    cudaGraphExecDestroy(ge);
    CSSG_CUDA(cudaMemcpyAsync(h.data(), dst, sizeof(FireState) * K, cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaStreamSynchronize(st));
    CSSG_CUDA(cudaGetLastError());
    if (result_host)
        for (int k = 0; k < K; ++k) {
            result_host[5 * k] = h[k].iterations;
            result_host[5 * k + 1] = h[k].forceMax;
            result_host[5 * k + 2] = h[k].dt;
            result_host[5 * k + 3] = h[k].alpha;
            result_host[5 * k + 4] = h[k].nSince;
        }
    return CSSG_OK;
}

namespace {
// gradientDescent::performUpdate's displacement (gradientDescent.cpp:12-16): deltaT * force, per component
__global__ void gd_displacement(int n3, const double* __restrict__ f, double* __restrict__ disp, double dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n3) disp[i] = dt * f[i];
}
}  // namespace

extern "C" int cssg_system_gradient_descent(cssg_system* s, int steps, double delta_t, int transport_velocity)
{
    if (!s || steps < 0 || !(delta_t >= 0)) return cssg_bad_args("cssg_system_gradient_descent");
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    s->eventsUsed = 0;
    for (int k = 0; k < steps; ++k) {
        launch_forces(s);
        gd_displacement<<<(3 * n + 255) / 256, 256, 0, st>>>(3 * n, s->force, s->disp, delta_t);
        cssg_launch_transport(s->dmeshes, s->sysOf, n, s->face, s->bary, s->disp, transport_velocity ? s->vel : nullptr,
                              transport_velocity ? 1 : 0, s->walkStatus, s->counters, s->pos, st, nullptr,
                              s->statusBits);
    }
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}

extern "C" int cssg_system_stress(cssg_system* s, double* stress_host)
{
    if (!s || !stress_host || s->K != 1) {
        cssg_set_error("cssg_system_stress: bad arguments (one system per call object)");
        return CSSG_ERR_ARG;
    }
    DeviceScope scope(s->ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    const int nBlocks = (n + 255) / 256;
    if (!s->pairD) {
        int cnt = 0;
        if (int rc = cssg_system_pairs(s, 0, nullptr, nullptr, nullptr, nullptr, &cnt)) return rc;
    }
    if (!s->stressPartials)
        if (int rc = alloc((void**)&s->stressPartials, sizeof(double) * 18 * (size_t)nBlocks + 16)) return rc;
    // simulation::computeMonodisperseStress calls findNeighbors on the current positions first
    launch_forces(s);
    int* overflow = (int*)(s->stressPartials + 18 * (size_t)nBlocks);
    CSSG_CUDA(cudaMemsetAsync(overflow, 0, sizeof(int), st));
    stress_partials<<<nBlocks, 256, 0, st>>>(n, s->pairCap, s->pairCount, s->pairD, s->pairT, s->vel, s->dsys,
                                             s->stressPartials, overflow);
    std::vector<double> part(18 * (size_t)nBlocks);
    int ovf = 0;
    CSSG_CUDA(cudaMemcpyAsync(part.data(), s->stressPartials, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaMemcpyAsync(&ovf, overflow, sizeof(int), cudaMemcpyDeviceToHost, st));
    CSSG_CUDA(cudaStreamSynchronize(st));
    if (ovf) {
        cssg_set_error("cssg_system_stress: a source has more candidate pairs than the pair buffer holds");
        return CSSG_ERR_CAPACITY;
    }
    double acc[18] = {0};
    for (int b = 0; b < nBlocks; ++b)
        for (int k = 0; k < 18; ++k) acc[k] += part[18 * b + k];
    const double area = s->meshes[0]->area;
    const double density = n / area;
    for (int k = 0; k < 9; ++k) stress_host[k] = density * 1.0 * acc[9 + k] / (2 * n) + acc[k] / (2 * 2 * area * n);
    return CSSG_OK;
}
