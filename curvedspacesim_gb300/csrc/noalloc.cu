// cssg_distance_batch_noalloc: cssg_distance_batch with every scratch buffer in fixed, file-scope device memory.
//
// For callers that must not allocate device memory during the call (a host code that has reserved the device's
// memory up front, or one that forbids allocator calls once its setup phase ends).  The propagation kernels, the
// table sizing and the results are those of cssg_distance_batch; only where the scratch lives differs:
//   * g_scratch holds the per-warp propagation slots (CSSG_NOALLOC_SCRATCH_BYTES); a call whose single slot would
//     not fit is rejected with CSSG_ERR_CAPACITY, and a call that fits fewer slots than it would otherwise use
//     runs with fewer slots (less parallelism, same results);
//   * g_sys, g_work and g_maxTargets hold the system descriptor, the persistent kernel's work counter and the
//     largest candidate count.
// Their device addresses come from cudaGetSymbolAddress once per device (first call on that device) and are kept.
// No call here allocates or frees device or pinned memory.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "cssg_internal.cuh"

namespace {

constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_scratch[CSSG_NOALLOC_SCRATCH_BYTES];
__device__ __align__(256) unsigned char g_sys[sizeof(SysDesc)];
__device__ __align__(16) int g_work;
__device__ __align__(16) int g_maxTargets;

struct Symbols {
    bool ready = false;
    unsigned char* scratch = nullptr;
    SysDesc* sys = nullptr;
    int* work = nullptr;
    int* maxTargets = nullptr;
};
Symbols g_symbols[kMaxDevices];
std::mutex g_symbolsMutex;

int symbols_for(int device, Symbols& out)
{
    if (device < 0 || device >= kMaxDevices) {
        cssg_set_error("cssg_distance_batch_noalloc: device index out of range");
        return CSSG_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_symbolsMutex);
    Symbols& s = g_symbols[device];
    if (!s.ready) {
        void* p = nullptr;
        CSSG_CUDA(cudaGetSymbolAddress(&p, g_scratch));
        s.scratch = (unsigned char*)p;
        CSSG_CUDA(cudaGetSymbolAddress(&p, g_sys));
        s.sys = (SysDesc*)p;
        CSSG_CUDA(cudaGetSymbolAddress(&p, g_work));
        s.work = (int*)p;
        CSSG_CUDA(cudaGetSymbolAddress(&p, g_maxTargets));
        s.maxTargets = (int*)p;
        if (((uintptr_t)s.scratch & 255) != 0) {
            cssg_set_error("cssg_distance_batch_noalloc: scratch symbol is not 256-byte aligned");
            return CSSG_ERR_CUDA;
        }
        s.ready = true;
    }
    out = s;
    return CSSG_OK;
}

// largest candidate count over the sources (one block)
__global__ void max_targets_kernel(int n, const int* __restrict__ off, int* __restrict__ out)
{
    int m = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = max(m, off[i + 1] - off[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ int part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        int r = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r = max(r, part[k]);
        *out = r;
    }
}

}  // namespace

extern "C" int cssg_distance_batch_noalloc(cssg_ctx* ctx, const cssg_mesh* mesh, int nSrc, const int* src_face,
                                           const double* src_bary, const int* cand_offsets, const int* cand_face,
                                           const double* cand_bary, int submesh, double max_dist,
                                           const double* threshold, double cutoff, double* d_out, double* tstart_out,
                                           double* tend_out, int* status, long long* stats)
{
    if (!ctx || !mesh || nSrc < 0 || (nSrc > 0 && (!src_face || !src_bary || !cand_offsets || !d_out || !status))) {
        cssg_set_error("cssg_distance_batch_noalloc: bad arguments");
        return CSSG_ERR_ARG;
    }
    if (nSrc == 0) return CSSG_OK;
    // everything below (the symbol lookup included) runs on the context's device, whatever device the calling
    // thread had selected; the caller's device is restored on return
    DeviceScope scope(ctx->device);
    CSSG_CUDA(scope.err);
    Symbols sym;
    if (int rc = symbols_for(ctx->device, sym)) return rc;
    cudaStream_t s = ctx->stream;

    max_targets_kernel<<<1, 1024, 0, s>>>(nSrc, cand_offsets, sym.maxTargets);
    int hmax = 0;
    CSSG_CUDA(cudaMemcpyAsync(&hmax, sym.maxTargets, sizeof(int), cudaMemcpyDeviceToHost, s));
    CSSG_CUDA(cudaStreamSynchronize(s));

    // table capacities: the sizing rule of cssg_distance_batch (one shared helper)
    const GeoSizing z = cssg_geo_sizing(mesh, hmax, submesh, max_dist, cutoff);
    const GeoCaps caps = z.caps;
    const size_t slotBytes = cssg_geo_slot_bytes(caps);
    if (slotBytes > (size_t)CSSG_NOALLOC_SCRATCH_BYTES) {
        cssg_set_error("cssg_distance_batch_noalloc: one propagation slot needs " + std::to_string(slotBytes) +
                       " bytes; the fixed scratch holds " + std::to_string((size_t)CSSG_NOALLOC_SCRATCH_BYTES) +
                       " (use cssg_distance_batch)");
        return CSSG_ERR_CAPACITY;
    }
    int sms = 0;
    CSSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    long long nSlots = std::min<long long>((long long)sms * 16, nSrc);
    nSlots = std::min<long long>(nSlots, (long long)(CSSG_NOALLOC_SCRATCH_BYTES / slotBytes));

    // what must start at zero / empty on every call: the work counter (memset) and every slot's tables
    // (initialisation kernel); the scratch keeps whatever the previous call left otherwise
    CSSG_CUDA(cudaMemsetAsync(sym.work, 0, sizeof(int), s));
    cssg_geo_init_scratch(sym.scratch, slotBytes, (int)nSlots, caps, s);
    SysDesc hd;
    memset(&hd, 0, sizeof(hd));
    hd.mesh = mesh->d;
    hd.searchMode = 0;
    hd.submesh = submesh;
    hd.maxDist = max_dist;
    hd.cutoff = cutoff;
    CSSG_CUDA(cudaMemcpyAsync(sym.sys, &hd, sizeof(SysDesc), cudaMemcpyHostToDevice, s));

    GeoLaunch L;
    memset(&L, 0, sizeof(L));
    L.sys = sym.sys;
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
    L.caps = caps;
    L.scratch = sym.scratch;
    L.slotBytes = slotBytes;
    L.nSlots = (int)nSlots;
    L.workCounter = sym.work;
    L.device = ctx->device;
    cssg_launch_geodesic(L, s);
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}
