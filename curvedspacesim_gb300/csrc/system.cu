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

// ---- cell list ------------------------------------------------------------------------------------------------
struct Grid {
    int nc[3];
    double cs[3];
    double lo[3];
};

__global__ void cell_assign(int n, const double* __restrict__ pos, Grid G, int* __restrict__ cellOf,
                            int* __restrict__ count)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int ci[3];
    for (int c = 0; c < 3; ++c) {
        int q = (int)floor((pos[3 * i + c] - G.lo[c]) / G.cs[c]);
        ci[c] = max(0, min(G.nc[c] - 1, q));
    }
    int cell = ci[0] + G.nc[0] * (ci[1] + G.nc[1] * ci[2]);
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
__global__ void nve_first_half(int n, double* __restrict__ v, const double* __restrict__ f, double* __restrict__ disp,
                               double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    disp[i] = dt * v[i] + 0.5 * dt * dt * f[i];
    v[i] += 0.5 * dt * f[i];
}

__global__ void nve_second_half(int n, double* __restrict__ v, const double* __restrict__ f, double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    v[i] += 0.5 * dt * f[i];
}

// chain layout: (M+1) x {pos, vel, accel, mass}, then kineticEnergy, scale
__global__ void nh_chain(double* ch, int Mc, double T, double dt, const double* partials, int nPartials)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double* bv = ch;
    double& KE = ch[4 * (Mc + 1)];
    double& scale = ch[4 * (Mc + 1) + 1];
    if (partials) {
        double s = 0;
        for (int b = 0; b < nPartials; ++b) s += partials[b];
        KE = s;
    }
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

__global__ void nvt_scale(int n, double* __restrict__ v, const double* __restrict__ ch, int Mc,
                          double* __restrict__ disp, double dt2)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    double s = ch[4 * (Mc + 1) + 1];
    v[i] = s * v[i];
    if (disp) disp[i] = dt2 * v[i];
}

__global__ void __launch_bounds__(KE_BLOCK) nvt_kick(int n, double* __restrict__ v, const double* __restrict__ f,
                                                     double* __restrict__ disp, double dt, double dt2,
                                                     double* __restrict__ partials)
{
    __shared__ double s[KE_BLOCK];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double ke = 0;
    if (i < n) {
        double vv[3];
        for (int c = 0; c < 3; ++c) {
            vv[c] = v[3 * i + c] + (dt / 1.0) * f[3 * i + c];
            v[3 * i + c] = vv[c];
            disp[3 * i + c] = dt2 * vv[c];
        }
        ke = 0.5 * 1.0 * (vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
    }
    s[threadIdx.x] = ke;
    __syncthreads();
    for (int o = KE_BLOCK / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = s[0];
}

__global__ void status_or(int n, const int* __restrict__ st, int* __restrict__ bits)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int b = (i < n && st[i]) ? (1 << st[i]) : 0;
    for (int o = 16; o > 0; o >>= 1) b |= __shfl_xor_sync(0xffffffffu, b, o);
    if ((threadIdx.x & 31) == 0 && b) atomicOr(bits, b);
}

int next_pow2(long long x)
{
    int p = 1;
    while (p < x && p < (1 << 30)) p <<= 1;
    return p;
}

}  // namespace

struct cssg_system {
    cssg_ctx* ctx;
    const cssg_mesh* mesh;
    int n;
    cssg_params P;
    // state
    int* face = nullptr;
    double* bary = nullptr;
    double* vel = nullptr;
    double* force = nullptr;
    double* disp = nullptr;
    double* pos = nullptr;
    int* walkStatus = nullptr;
    int* srcStatus = nullptr;
    int* statusBits = nullptr;           // device: OR of 1 << status over walks and sources
    unsigned long long* counters = nullptr;  // device: crossings, windows, launches, in-range pairs, capacity hits
    // cell list
    bool useCells = false;
    Grid grid;
    int totalCells = 0;
    int* cellOf = nullptr;
    int* cellCount = nullptr;
    int* cellStart = nullptr;
    int* cellCursor = nullptr;
    int* cellList = nullptr;
    int* slotOf = nullptr;
    int* scanBlocks = nullptr;
    int nScanBlocks = 0;
    // geodesic scratch (regular and retry passes)
    GeoCaps caps, bigCaps;
    void* scratch = nullptr;
    void* bigScratch = nullptr;
    size_t slotBytes = 0, bigSlotBytes = 0;
    int nSlots = 0, nBigSlots = 0;
    int* work = nullptr;  // [0] work counter, [1] retry work counter, [2] failure count
    int* failList = nullptr;
    // pair output
    int pairCap = 0;
    double* pairD = nullptr;
    double* pairT = nullptr;
    int* pairJ = nullptr;
    int* pairCount = nullptr;
    // NVT
    double* chain = nullptr;
    double* kePartials = nullptr;
    int nKeBlocks = 0;
    // graph
    cudaGraphExec_t graphExec = nullptr;
    // timing
    bool timing = false;
    std::vector<cudaEvent_t> events;
    int eventsUsed = 0;
    double lastMs[4] = {0, 0, 0, 0};
};

namespace {

int alloc(void** p, size_t bytes)
{
    CSSG_CUDA(cudaMalloc(p, bytes ? bytes : 16));
    return CSSG_OK;
}

int record(cssg_system* s, int slot)
{
    if (!s->timing) return -1;
    if (s->eventsUsed >= (int)s->events.size()) return -1;
    int k = s->eventsUsed++;
    cudaEventRecord(s->events[k], s->ctx->stream);
    (void)slot;
    return k;
}

// findNeighbors + computeForces into s->force
void launch_forces(cssg_system* s)
{
    cudaStream_t st = s->ctx->stream;
    const DevMesh& M = s->mesh->d;
    const int n = s->n;
    const int tb = 256;
    if (s->useCells) {
        cudaMemsetAsync(s->cellCount, 0, sizeof(int) * (s->totalCells + 1), st);
        cudaMemsetAsync(s->cellCursor, 0, sizeof(int) * s->totalCells, st);
        cell_assign<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->pos, s->grid, s->cellOf, s->cellCount);
        scan_local<<<s->nScanBlocks, SCAN_BLOCK, 0, st>>>(s->cellCount, s->totalCells, s->cellStart, s->scanBlocks);
        scan_blocks<<<1, 1024, 0, st>>>(s->scanBlocks, s->nScanBlocks, s->cellStart + s->totalCells);
        scan_add<<<(s->totalCells + 255) / 256, 256, 0, st>>>(s->cellStart, s->totalCells, s->scanBlocks);
        cell_scatter<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->cellOf, s->cellStart, s->cellCursor, s->cellList,
                                                       s->slotOf);
        cell_sort<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->cellOf, s->cellStart, s->slotOf, s->cellList);
    }
    cudaMemsetAsync(s->work, 0, 3 * sizeof(int), st);
    GeoLaunch L;
    memset(&L, 0, sizeof(L));
    L.nSrc = n;
    L.srcFace = s->face;
    L.srcBary = s->bary;
    L.srcPos = s->pos;
    L.order = s->useCells ? s->cellList : nullptr;
    L.searchMode = s->useCells ? 1 : 2;
    L.nPart = n;
    L.partFace = s->face;
    L.partBary = s->bary;
    L.partPos = s->pos;
    L.cellStart = s->cellStart;
    L.cellList = s->cellList;
    for (int c = 0; c < 3; ++c) {
        L.nc[c] = s->grid.nc[c];
        L.cs[c] = s->grid.cs[c];
    }
    L.range2 = s->P.range * s->P.range;
    L.submesh = s->P.submesh;
    L.maxDist = s->P.max_dist;
    L.cutoff = s->P.cutoff;
    L.dOut = s->pairD;
    L.tsOut = s->pairT;
    L.pairJ = s->pairJ;
    L.pairCount = s->pairCount;
    L.pairCap = s->pairCap;
    L.force = s->force;
    L.forceKind = s->P.force_kind;
    L.k = s->P.k;
    L.sigma = s->P.sigma;
    L.status = s->srcStatus;
    L.counters = s->counters + 1;
    L.delta = 1e300;
    L.maxRounds = 1 << 16;
    L.caps = s->caps;
    L.scratch = s->scratch;
    L.slotBytes = s->slotBytes;
    L.nSlots = s->nSlots;
    L.workCounter = s->work;
    L.failList = s->failList;
    L.failCount = s->work + 2;
    int e0 = record(s, 0);
    cssg_launch_geodesic(M, L, (s->nSlots + 7) / 8, st);
    // retry pass with large tables for the sources whose tables overflowed (usually none: exits at once)
    GeoLaunch R = L;
    R.caps = s->bigCaps;
    R.scratch = s->bigScratch;
    R.slotBytes = s->bigSlotBytes;
    R.nSlots = s->nBigSlots;
    R.workCounter = s->work + 1;
    R.order = s->failList;
    R.itemCountDev = s->work + 2;
    R.failList = nullptr;
    R.failCount = nullptr;
    cssg_launch_geodesic(M, R, (s->nBigSlots + 7) / 8, st);
    int e1 = record(s, 1);
    status_or<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->srcStatus, s->statusBits);
    (void)e0;
    (void)e1;
}

void launch_walk(cssg_system* s)
{
    cudaStream_t st = s->ctx->stream;
    int e0 = record(s, 2);
    cssg_launch_transport(s->mesh->d, s->n, s->face, s->bary, s->disp, s->vel, 1, s->walkStatus, s->counters,
                          s->pos, st);
    int e1 = record(s, 3);
    status_or<<<(s->n + 255) / 256, 256, 0, st>>>(s->n, s->walkStatus, s->statusBits);
    (void)e0;
    (void)e1;
}

void launch_step(cssg_system* s)
{
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    const int tb = 256;
    const double dt = s->P.dt;
    if (s->P.integrator == 0) {
        nve_first_half<<<(3 * n + tb - 1) / tb, tb, 0, st>>>(n, s->vel, s->force, s->disp, dt);
        launch_walk(s);
        launch_forces(s);
        nve_second_half<<<(3 * n + tb - 1) / tb, tb, 0, st>>>(n, s->vel, s->force, dt);
    } else {
        const int Mc = s->P.chain_length;
        const double T = s->P.temperature;
        nh_chain<<<1, 32, 0, st>>>(s->chain, Mc, T, dt, nullptr, 0);
        nvt_scale<<<(3 * n + tb - 1) / tb, tb, 0, st>>>(n, s->vel, s->chain, Mc, s->disp, 0.5 * dt);
        launch_walk(s);
        launch_forces(s);
        nvt_kick<<<s->nKeBlocks, KE_BLOCK, 0, st>>>(n, s->vel, s->force, s->disp, dt, 0.5 * dt, s->kePartials);
        launch_walk(s);
        nh_chain<<<1, 32, 0, st>>>(s->chain, Mc, T, dt, s->kePartials, s->nKeBlocks);
        nvt_scale<<<(3 * n + tb - 1) / tb, tb, 0, st>>>(n, s->vel, s->chain, Mc, nullptr, 0.0);
    }
}

int reset_chain(cssg_system* s)
{
    int Mc = s->P.chain_length;
    std::vector<double> h(4 * (Mc + 1) + 2, 0.0);
    double T = s->P.temperature, tau = s->P.tau;
    h[3] = 2.0 * (s->n - 1) * T * tau * tau;
    for (int ii = 1; ii < Mc + 1; ++ii) h[4 * ii + 3] = T * tau * tau;
    h[4 * (Mc + 1)] = h[3];
    h[4 * (Mc + 1) + 1] = 1.0;
    CSSG_CUDA(cudaMemcpyAsync(s->chain, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s->ctx->stream));
    CSSG_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return CSSG_OK;
}

}  // namespace

extern "C" int cssg_system_create(cssg_ctx* ctx, const cssg_mesh* mesh, int n, const cssg_params* params,
                                  cssg_system** out)
{
    if (!ctx || !mesh || !params || !out || n <= 0) {
        cssg_set_error("cssg_system_create: bad arguments");
        return CSSG_ERR_ARG;
    }
    const cssg_params& P = *params;
    if (P.integrator < 0 || P.integrator > 1 || P.force_kind < 0 || P.force_kind > 1 || !(P.dt > 0) ||
        (P.integrator == 1 && P.chain_length < 1) || !(P.cutoff > 0)) {
        cssg_set_error("cssg_system_create: bad parameters");
        return CSSG_ERR_ARG;
    }
    CSSG_CUDA(cudaSetDevice(ctx->device));
    cssg_system* s = new cssg_system();
    s->ctx = ctx;
    s->mesh = mesh;
    s->n = n;
    s->P = P;
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
    TRY(alloc((void**)&s->work, sizeof(int) * 4));
    TRY(alloc((void**)&s->failList, sizeof(int) * n));
    cudaMemset(s->force, 0, sizeof(double) * 3 * n);
    cudaMemset(s->vel, 0, sizeof(double) * 3 * n);
    cudaMemset(s->face, 0, sizeof(int) * n);
    cudaMemset(s->statusBits, 0, sizeof(int));
    cudaMemset(s->counters, 0, sizeof(unsigned long long) * 8);
    // cell list over the reference's domain: cells of size >= range (hyperRectangularCellList::setGridSize)
    s->useCells = P.range > 0;
    if (s->useCells) {
        long long total = 1;
        for (int c = 0; c < 3; ++c) {
            double ext = mesh->d.bbMax[c] - mesh->d.bbMin[c];
            s->grid.nc[c] = std::max(1, (int)std::floor(ext / P.range));
            s->grid.cs[c] = ext / s->grid.nc[c];
            s->grid.lo[c] = mesh->d.bbMin[c];
            total *= s->grid.nc[c];
        }
        if (total > (1LL << 28)) {
            cssg_set_error("cssg_system_create: cell grid too large for the interaction range");
            cssg_system_destroy(s);
            return CSSG_ERR_CAPACITY;
        }
        s->totalCells = (int)total;
        s->nScanBlocks = (int)((total + SCAN_BLOCK * SCAN_ITEMS - 1) / (SCAN_BLOCK * SCAN_ITEMS));
        TRY(alloc((void**)&s->cellOf, sizeof(int) * n));
        TRY(alloc((void**)&s->cellCount, sizeof(int) * (total + 1)));
        TRY(alloc((void**)&s->cellStart, sizeof(int) * (total + 1)));
        TRY(alloc((void**)&s->cellCursor, sizeof(int) * total));
        TRY(alloc((void**)&s->cellList, sizeof(int) * n));
        TRY(alloc((void**)&s->slotOf, sizeof(int) * n));
        TRY(alloc((void**)&s->scanBlocks, sizeof(int) * (s->nScanBlocks + 1)));
    } else {
        for (int c = 0; c < 3; ++c) {
            s->grid.nc[c] = 1;
            s->grid.cs[c] = 1;
            s->grid.lo[c] = 0;
        }
    }
    // table sizes from the expected neighbourhood: faces within the cutoff and candidates within the range
    double reach = P.cutoff;
    if (P.submesh && P.max_dist < reach) reach = P.max_dist;
    long long estF = (long long)(3.14159265 * reach * reach / mesh->meanFaceArea * 2.0) + 48;
    if (estF > mesh->d.nF) estF = mesh->d.nF;
    double density = n / mesh->area;
    long long estT = P.range > 0 ? (long long)(density * 3.14159265 * P.range * P.range) : n;
    s->caps.CT = (int)std::min<long long>(std::max<long long>(64, 6 * estT + 32), std::max(64, n));
    s->caps.CF = next_pow2(2 * (estF + s->caps.CT) + 32);
    s->caps.CV = next_pow2(2 * estF + 64);
    s->caps.CW = (int)(8 * estF + 256);
    s->caps.CL = (int)(estF + 128);
    s->caps.CLOG = (int)(4 * s->caps.CT + 2 * estF + 256);
    s->bigCaps.CT = std::max(s->caps.CT * 8, std::min(n, 4096));
    s->bigCaps.CF = next_pow2(16LL * s->caps.CF);
    s->bigCaps.CV = next_pow2(16LL * s->caps.CV);
    s->bigCaps.CW = 16 * s->caps.CW;
    s->bigCaps.CL = 16 * s->caps.CL;
    s->bigCaps.CLOG = 16 * s->caps.CLOG + 8 * s->bigCaps.CT;
    s->slotBytes = cssg_geo_slot_bytes(s->caps);
    s->bigSlotBytes = cssg_geo_slot_bytes(s->bigCaps);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    s->nSlots = std::min(n, sms * 32);
    s->nSlots = ((s->nSlots + 7) / 8) * 8;
    s->nBigSlots = std::min(n, sms);
    TRY(alloc(&s->scratch, s->slotBytes * (size_t)s->nSlots));
    TRY(alloc(&s->bigScratch, s->bigSlotBytes * (size_t)s->nBigSlots));
    cssg_geo_init_scratch(s->scratch, s->slotBytes, s->nSlots, s->caps, ctx->stream);
    cssg_geo_init_scratch(s->bigScratch, s->bigSlotBytes, s->nBigSlots, s->bigCaps, ctx->stream);
    // NVT
    int Mc = std::max(1, P.chain_length);
    TRY(alloc((void**)&s->chain, sizeof(double) * (4 * (Mc + 1) + 2)));
    s->nKeBlocks = (n + KE_BLOCK - 1) / KE_BLOCK;
    TRY(alloc((void**)&s->kePartials, sizeof(double) * s->nKeBlocks));
    if (P.integrator == 1) TRY(reset_chain(s));
    CSSG_CUDA(cudaStreamSynchronize(ctx->stream));
    CSSG_CUDA(cudaGetLastError());
#undef TRY
    *out = s;
    return CSSG_OK;
}

extern "C" int cssg_system_destroy(cssg_system* s)
{
    if (!s) return CSSG_OK;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    if (s->graphExec) cudaGraphExecDestroy(s->graphExec);
    for (cudaEvent_t e : s->events) cudaEventDestroy(e);
    void* ptrs[] = {s->face, s->bary, s->vel, s->force, s->disp, s->pos, s->walkStatus, s->srcStatus,
                    s->statusBits, s->counters, s->cellOf, s->cellCount, s->cellStart, s->cellCursor, s->cellList,
                    s->slotOf, s->scanBlocks, s->scratch, s->bigScratch, s->work, s->failList, s->pairD, s->pairT, s->pairJ,
                    s->pairCount, s->chain, s->kePartials};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete s;
    return CSSG_OK;
}

extern "C" int cssg_system_set_state(cssg_system* s, const int* face, const double* bary, const double* vel,
                                     const double* force)
{
    if (!s) return CSSG_ERR_ARG;
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    if (face) {
        for (int i = 0; i < n; ++i)
            if (face[i] < 0 || face[i] >= s->mesh->d.nF) {
                cssg_set_error("cssg_system_set_state: face index out of range");
                return CSSG_ERR_ARG;
            }
        CSSG_CUDA(cudaMemcpyAsync(s->face, face, sizeof(int) * n, cudaMemcpyHostToDevice, st));
    }
    if (bary) CSSG_CUDA(cudaMemcpyAsync(s->bary, bary, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (vel) CSSG_CUDA(cudaMemcpyAsync(s->vel, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    if (force) CSSG_CUDA(cudaMemcpyAsync(s->force, force, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    cssg_launch_positions(s->mesh->d, n, s->face, s->bary, s->pos, st);
    CSSG_CUDA(cudaStreamSynchronize(st));
    return CSSG_OK;
}

extern "C" int cssg_system_reset_thermostat(cssg_system* s)
{
    if (!s) return CSSG_ERR_ARG;
    return reset_chain(s);
}

extern "C" int cssg_system_kernels_per_step(cssg_system* s, int* count)
{
    if (!s || !count) return CSSG_ERR_ARG;
    // walk + status_or ; [cell list: assign, scan x3, scatter, sort] + geodesic + retry + status_or
    int walk = 2, forces = (s->useCells ? 6 : 0) + 3;
    *count = s->P.integrator == 0 ? (1 + walk + forces + 1) : (2 + walk + forces + 1 + walk + 2);
    return CSSG_OK;
}

extern "C" int cssg_system_get_state(cssg_system* s, int* face, double* bary, double* vel, double* force)
{
    if (!s) return CSSG_ERR_ARG;
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
    if (!s) return CSSG_ERR_ARG;
    if (face) *face = s->face;
    if (bary) *bary = s->bary;
    if (vel) *vel = s->vel;
    if (force) *force = s->force;
    return CSSG_OK;
}

extern "C" int cssg_system_step(cssg_system* s, int steps, int use_graph)
{
    if (!s || steps < 0) return CSSG_ERR_ARG;
    cudaStream_t st = s->ctx->stream;
    s->eventsUsed = 0;
    if (use_graph && !s->timing) {
        if (!s->graphExec) {
            cudaGraph_t g;
            CSSG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            launch_step(s);
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (e != cudaSuccess) return cssg_cuda_fail(e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&s->graphExec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                s->graphExec = nullptr;
                return cssg_cuda_fail(e, "cudaGraphInstantiate");
            }
        }
        for (int k = 0; k < steps; ++k) CSSG_CUDA(cudaGraphLaunch(s->graphExec, st));
    } else {
        if (s->timing) {
            size_t need = (size_t)steps * 6 + 8;
            while (s->events.size() < need) {
                cudaEvent_t e;
                CSSG_CUDA(cudaEventCreate(&e));
                s->events.push_back(e);
            }
        }
        for (int k = 0; k < steps; ++k) launch_step(s);
    }
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}

extern "C" int cssg_system_compute_forces(cssg_system* s)
{
    if (!s) return CSSG_ERR_ARG;
    s->eventsUsed = 0;
    launch_forces(s);
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}

extern "C" int cssg_system_check(cssg_system* s, int* bits, unsigned long long* counters)
{
    if (!s) return CSSG_ERR_ARG;
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
    if (!s) return CSSG_ERR_ARG;
    cudaStream_t st = s->ctx->stream;
    if (!s->pairD) {
        // enable pair output for subsequent force evaluations
        s->pairCap = std::max(16, s->caps.CT);
        size_t slots = (size_t)s->n * s->pairCap;
        int rc;
        if ((rc = alloc((void**)&s->pairD, sizeof(double) * slots)) || (rc = alloc((void**)&s->pairT, sizeof(double) * 3 * slots)) ||
            (rc = alloc((void**)&s->pairJ, sizeof(int) * slots)) || (rc = alloc((void**)&s->pairCount, sizeof(int) * s->n)))
            return rc;
        if (s->graphExec) {
            cudaGraphExecDestroy(s->graphExec);
            s->graphExec = nullptr;
        }
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
    if (!s || !chain) return CSSG_ERR_ARG;
    int Mc = std::max(1, s->P.chain_length);
    int len = 4 * (Mc + 1) + 2;
    if (capacity < len) {
        cssg_set_error("cssg_system_chain: capacity too small");
        return CSSG_ERR_CAPACITY;
    }
    CSSG_CUDA(cudaMemcpyAsync(chain, s->chain, sizeof(double) * len, cudaMemcpyDeviceToHost, s->ctx->stream));
    CSSG_CUDA(cudaStreamSynchronize(s->ctx->stream));
    return CSSG_OK;
}

extern "C" int cssg_system_timing(cssg_system* s, int enable)
{
    if (!s) return CSSG_ERR_ARG;
    s->timing = enable != 0;
    return CSSG_OK;
}

// ms[0] = geodesic/force kernel total, ms[1] = walk kernel total over the last step() call
extern "C" int cssg_system_last_times(cssg_system* s, double* ms, int capacity)
{
    if (!s || !ms || capacity < 2) return CSSG_ERR_ARG;
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
