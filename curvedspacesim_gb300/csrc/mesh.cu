// Mesh upload, contexts and error plumbing of libcssg.so.
//
// cssg_mesh_create replaces triangulatedMeshSpace::loadMeshFromFile / updateMeshSpanAndTree
// (src/models/triangulatedMeshSpace.cpp:6-72): instead of a CGAL Surface_mesh plus AABB tree it builds, once on the
// host, the flat arrays the kernels read - neighbour-across-edge table, per-edge 2D frames, vertex -> face lists,
// clockwise vertex rings (the order CGAL's vertex circulator visits, which throughVertex depends on), angle sums
// and the bounding box (origin included, like the reference's span computation).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "cssg_internal.cuh"

static thread_local std::string g_lastError;

void cssg_set_error(const std::string& msg) { g_lastError = msg; }

int cssg_bad_args(const char* fn)
{
    g_lastError = std::string(fn) + ": bad arguments (null handle or pointer, or a value out of range)";
    return CSSG_ERR_ARG;
}

int cssg_cuda_fail(cudaError_t e, const char* what)
{
    g_lastError = std::string(what) + ": " + cudaGetErrorString(e);
    return CSSG_ERR_CUDA;
}

extern "C" const char* cssg_last_error(void) { return g_lastError.c_str(); }
extern "C" const char* cssg_version(void) { return "cssg 0.1 (sm_103a)"; }

namespace {

inline double twoPiConst() { return 6.283185307179586; }

template <typename T>
int upload(const std::vector<T>& h, T** d, void** keep)
{
    size_t bytes = h.size() * sizeof(T);
    if (bytes == 0) bytes = sizeof(T);
    CSSG_CUDA(cudaMalloc((void**)d, bytes));
    if (!h.empty()) CSSG_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    *keep = *d;
    return CSSG_OK;
}

}  // namespace

extern "C" int cssg_mesh_create(const double* V, int nV, const int* F, int nF, int device, cssg_mesh** out)
{
    if (!V || !F || !out || nV <= 0 || nF <= 0) {
        cssg_set_error("cssg_mesh_create: empty mesh or null pointer");
        return CSSG_ERR_ARG;
    }
    for (int i = 0; i < 3 * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) {
            cssg_set_error("cssg_mesh_create: face index out of range");
            return CSSG_ERR_ARG;
        }
    CSSG_CUDA(cudaSetDevice(device));
    std::vector<int> twin(3 * (size_t)nF, -1);
    {
        std::unordered_map<uint64_t, int> edge;
        edge.reserve(3 * (size_t)nF);
        for (int f = 0; f < nF; ++f)
            for (int k = 0; k < 3; ++k) {
                uint64_t a = (uint32_t)F[3 * f + k], b = (uint32_t)F[3 * f + (k + 1) % 3];
                if (!edge.emplace((a << 32) | b, 3 * f + k).second) {
                    cssg_set_error("cssg_mesh_create: non-manifold or inconsistently oriented edge");
                    return CSSG_ERR_ARG;
                }
            }
        for (int f = 0; f < nF; ++f)
            for (int k = 0; k < 3; ++k) {
                uint64_t a = (uint32_t)F[3 * f + k], b = (uint32_t)F[3 * f + (k + 1) % 3];
                auto it = edge.find((b << 32) | a);
                if (it != edge.end()) twin[3 * f + k] = it->second;
            }
    }
    std::vector<double> N(3 * (size_t)nF), geom(9 * (size_t)nF);
    double area = 0, edgeSum = 0;
    for (int f = 0; f < nF; ++f) {
        const double* p0 = &V[3 * F[3 * f]];
        const double* p1 = &V[3 * F[3 * f + 1]];
        const double* p2 = &V[3 * F[3 * f + 2]];
        double e1[3], e2[3], n[3];
        for (int c = 0; c < 3; ++c) {
            e1[c] = p1[c] - p0[c];
            e2[c] = p2[c] - p0[c];
        }
        n[0] = e1[1] * e2[2] - e1[2] * e2[1];
        n[1] = e1[2] * e2[0] - e1[0] * e2[2];
        n[2] = e1[0] * e2[1] - e1[1] * e2[0];
        double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (!(nn > 0)) {
            cssg_set_error("cssg_mesh_create: degenerate (zero-area) face");
            return CSSG_ERR_ARG;
        }
        area += 0.5 * nn;
        for (int c = 0; c < 3; ++c) N[3 * f + c] = n[c] / nn;
        for (int k = 0; k < 3; ++k) {
            const double* A = &V[3 * F[3 * f + k]];
            const double* B = &V[3 * F[3 * f + (k + 1) % 3]];
            const double* C = &V[3 * F[3 * f + (k + 2) % 3]];
            double ab[3], ac[3];
            for (int c = 0; c < 3; ++c) {
                ab[c] = B[c] - A[c];
                ac[c] = C[c] - A[c];
            }
            double L = std::sqrt(ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2]);
            double cr0 = ab[1] * ac[2] - ab[2] * ac[1], cr1 = ab[2] * ac[0] - ab[0] * ac[2],
                   cr2 = ab[0] * ac[1] - ab[1] * ac[0];
            geom[9 * f + 3 * k] = L;
            geom[9 * f + 3 * k + 1] = (ac[0] * ab[0] + ac[1] * ab[1] + ac[2] * ab[2]) / L;
            geom[9 * f + 3 * k + 2] = std::sqrt(cr0 * cr0 + cr1 * cr1 + cr2 * cr2) / L;
            edgeSum += L;
        }
    }
    std::vector<double> exitu(12 * (size_t)nF);
    for (int f = 0; f < nF; ++f)
        for (int k = 0; k < 3; ++k) {
            double L = geom[9 * f + 3 * k], cx = geom[9 * f + 3 * k + 1], cy = geom[9 * f + 3 * k + 2];
            double n1 = std::sqrt(cx * cx + cy * cy);
            double bx = L - cx, by = -cy;
            double n2 = std::sqrt(bx * bx + by * by);
            exitu[12 * f + 4 * k] = cx / n1;
            exitu[12 * f + 4 * k + 1] = cy / n1;
            exitu[12 * f + 4 * k + 2] = bx / n2;
            exitu[12 * f + 4 * k + 3] = by / n2;
        }
    std::vector<int> vfStart(nV + 1, 0), vfList(3 * (size_t)nF);
    for (int i = 0; i < 3 * nF; ++i) vfStart[F[i] + 1]++;
    for (int v = 0; v < nV; ++v) vfStart[v + 1] += vfStart[v];
    {
        std::vector<int> fill(vfStart.begin(), vfStart.end() - 1);
        for (int f = 0; f < nF; ++f)
            for (int k = 0; k < 3; ++k) vfList[fill[F[3 * f + k]]++] = f;
    }
    std::vector<unsigned char> vflag(nV, 0);
    std::vector<double> angle(nV, 0.0);
    for (int f = 0; f < nF; ++f)
        for (int k = 0; k < 3; ++k) {
            if (twin[3 * f + k] < 0) {
                vflag[F[3 * f + k]] |= VF_BORDER;
                vflag[F[3 * f + (k + 1) % 3]] |= VF_BORDER;
            }
            const double* A = &V[3 * F[3 * f + k]];
            const double* B = &V[3 * F[3 * f + (k + 1) % 3]];
            const double* C = &V[3 * F[3 * f + (k + 2) % 3]];
            double ab[3], ac[3], lab = 0, lac = 0, d = 0;
            for (int c = 0; c < 3; ++c) {
                ab[c] = B[c] - A[c];
                ac[c] = C[c] - A[c];
                lab += ab[c] * ab[c];
                lac += ac[c] * ac[c];
                d += ab[c] * ac[c];
            }
            double cs = d / std::sqrt(lab * lac);
            cs = cs > 1 ? 1 : (cs < -1 ? -1 : cs);
            angle[F[3 * f + k]] += std::acos(cs);
        }
    const double twoPi = 6.283185307179586;
    for (int v = 0; v < nV; ++v)
        if (angle[v] > twoPi + 1e-9) vflag[v] |= VF_SADDLE;
    // clockwise rings: from face f around v go to the face across the edge (v -> next of v in f)
    std::vector<int> ringStart(nV + 1, 0), ringV;
    ringV.reserve(6 * (size_t)nV);
    for (int v = 0; v < nV; ++v) {
        ringStart[v] = (int)ringV.size();
        if ((vflag[v] & VF_BORDER) || vfStart[v + 1] == vfStart[v]) continue;
        int f0 = vfList[vfStart[v]], f = f0, k = 0;
        while (F[3 * f + k] != v) ++k;
        size_t base = ringV.size();
        ringV.push_back(F[3 * f + (k + 2) % 3]);
        bool ok = true;
        for (int guard = 0;; ++guard) {
            ringV.push_back(F[3 * f + (k + 1) % 3]);
            int t = twin[3 * f + k];
            if (t < 0 || guard > 4096) { ok = false; break; }
            f = t / 3;
            k = 0;
            while (F[3 * f + k] != v) ++k;
            if (f == f0) break;
        }
        if (ok && (int)(ringV.size() - base - 1) == vfStart[v + 1] - vfStart[v]) {
            ringV.pop_back();
            vflag[v] |= VF_RING;
        } else {
            ringV.resize(base);  // pinched vertex: no single ring
        }
    }
    ringStart[nV] = (int)ringV.size();
    // ring starts must be monotone for vertices without a ring
    for (int v = nV - 1; v >= 0; --v)
        if (!(vflag[v] & VF_RING)) ringStart[v] = ringStart[v + 1];

    // per-face curvature features: mean curvature from the dihedral angles of its three edges
    // (H_f = sum_e theta_e L_e / (4 A_f), theta signed positive where the surface bends away from the normal) and
    // Gaussian curvature as the mean angle defect of its vertices over their barycentric areas
    std::vector<float> fcurv(3 * (size_t)nF, 0.0f);
    {
        std::vector<double> varea(nV, 0.0);
        for (int f = 0; f < nF; ++f) {
            double a = 0;
            for (int k = 0; k < 3; ++k) a = geom[9 * f + 3 * k] * geom[9 * f + 3 * k + 2] * 0.5;
            for (int k = 0; k < 3; ++k) varea[F[3 * f + k]] += a / 3.0;
        }
        for (int f = 0; f < nF; ++f) {
            double A = geom[9 * f] * geom[9 * f + 2] * 0.5;
            double H = 0, Kg = 0, el = 0;
            for (int k = 0; k < 3; ++k) {
                int t = twin[3 * f + k];
                double L = geom[9 * f + 3 * k];
                el += L / 3.0;
                if (t >= 0) {
                    int g = t / 3;
                    const double* n1 = &N[3 * f];
                    const double* n2 = &N[3 * g];
                    double c = n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2];
                    c = c > 1 ? 1 : (c < -1 ? -1 : c);
                    double th = std::acos(c);
                    // convex edge: the neighbour's far vertex lies below this face's plane
                    const double* q = &V[3 * F[3 * g + (t % 3 + 2) % 3]];
                    const double* p0 = &V[3 * F[3 * f + k]];
                    double side = (q[0] - p0[0]) * n1[0] + (q[1] - p0[1]) * n1[1] + (q[2] - p0[2]) * n1[2];
                    H += (side <= 0 ? th : -th) * L;
                }
                int v = F[3 * f + k];
                Kg += (twoPiConst() - angle[v]) / (varea[v] > 0 ? varea[v] : 1.0) / 3.0;
            }
            fcurv[3 * f] = (float)(H / (4.0 * A));
            fcurv[3 * f + 1] = (float)Kg;
            fcurv[3 * f + 2] = (float)el;
        }
    }

    cssg_mesh* m = new cssg_mesh();
    memset(m->buffers, 0, sizeof(m->buffers));
    m->device = device;
    m->area = area;
    m->meanEdge = edgeSum / (3.0 * nF);
    m->meanFaceArea = area / nF;
    DevMesh& d = m->d;
    d.nV = nV;
    d.nF = nF;
    for (int c = 0; c < 3; ++c) {
        d.bbMin[c] = 0;
        d.bbMax[c] = 0;
    }
    for (int v = 0; v < nV; ++v)
        for (int c = 0; c < 3; ++c) {
            d.bbMin[c] = std::min(d.bbMin[c], V[3 * v + c]);
            d.bbMax[c] = std::max(d.bbMax[c], V[3 * v + c]);
        }
    std::vector<double> hv(V, V + 3 * (size_t)nV);
    std::vector<int> hf(F, F + 3 * (size_t)nF);
    int rc = CSSG_OK;
    double *dV, *dN, *dG;
    int *dF, *dT, *dVS, *dVL, *dRS, *dRV;
    unsigned char* dVF;
    float* dFC;
    double* dEU;
    if ((rc = upload(hv, &dV, &m->buffers[0])) || (rc = upload(hf, &dF, &m->buffers[1])) ||
        (rc = upload(twin, &dT, &m->buffers[2])) || (rc = upload(N, &dN, &m->buffers[3])) ||
        (rc = upload(geom, &dG, &m->buffers[4])) || (rc = upload(vfStart, &dVS, &m->buffers[5])) ||
        (rc = upload(vfList, &dVL, &m->buffers[6])) || (rc = upload(ringStart, &dRS, &m->buffers[7])) ||
        (rc = upload(ringV, &dRV, &m->buffers[8])) || (rc = upload(vflag, &dVF, &m->buffers[9])) ||
        (rc = upload(fcurv, &dFC, &m->buffers[11])) || (rc = upload(exitu, &dEU, &m->buffers[12]))) {
        cssg_mesh_destroy(m);
        return rc;
    }
    d.V = dV;
    d.F = dF;
    d.twin = dT;
    d.N = dN;
    d.geom = dG;
    d.vfStart = dVS;
    d.vfList = dVL;
    d.ringStart = dRS;
    d.ringV = dRV;
    d.vflag = dVF;
    d.fcurv = dFC;
    d.exitu = dEU;
    d.bc = BC_CLOSED;
    {
        DevMesh* ds = nullptr;
        cudaError_t e = cudaMalloc((void**)&ds, sizeof(DevMesh));
        if (e == cudaSuccess) e = cudaMemcpy(ds, &d, sizeof(DevMesh), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cssg_mesh_destroy(m);
            return cssg_cuda_fail(e, "mesh descriptor upload");
        }
        m->dself = ds;
        m->buffers[10] = ds;
    }
    *out = m;
    return CSSG_OK;
}

extern "C" int cssg_mesh_destroy(cssg_mesh* m)
{
    if (!m) return CSSG_OK;
    cudaSetDevice(m->device);
    for (void* b : m->buffers)
        if (b) cudaFree(b);
    delete m;
    return CSSG_OK;
}

extern "C" int cssg_mesh_set_boundary(cssg_mesh* m, int bc)
{
    if (!m || bc < BC_CLOSED || bc > BC_ABSORBING) {
        cssg_set_error("cssg_mesh_set_boundary: bad arguments (0 closed, 1 tangential, 2 absorbing)");
        return CSSG_ERR_ARG;
    }
    m->d.bc = bc;
    CSSG_CUDA(cudaSetDevice(m->device));
    CSSG_CUDA(cudaMemcpy(&m->dself->bc, &bc, sizeof(int), cudaMemcpyHostToDevice));
    return CSSG_OK;
}

extern "C" int cssg_mesh_info(const cssg_mesh* m, int* nV, int* nF, double* area, double* bbox)
{
    if (!m) {
        cssg_set_error("cssg_mesh_info: null mesh");
        return CSSG_ERR_ARG;
    }
    if (nV) *nV = m->d.nV;
    if (nF) *nF = m->d.nF;
    if (area) *area = m->area;
    if (bbox)
        for (int c = 0; c < 3; ++c) {
            bbox[c] = m->d.bbMin[c];
            bbox[3 + c] = m->d.bbMax[c];
        }
    return CSSG_OK;
}

extern "C" int cssg_ctx_create(int device, void* stream, cssg_ctx** out)
{
    if (!out) {
        cssg_set_error("cssg_ctx_create: null out");
        return CSSG_ERR_ARG;
    }
    CSSG_CUDA(cudaSetDevice(device));
    {
        // the propagation kernels call out-of-line helpers and need close to 1 KB of stack per thread (ptxas
        // reports up to ~1000 bytes cumulative); give them headroom above the 1 KB default
        size_t stack = 0;
        CSSG_CUDA(cudaDeviceGetLimit(&stack, cudaLimitStackSize));
        if (stack < 4096) CSSG_CUDA(cudaDeviceSetLimit(cudaLimitStackSize, 4096));
    }
    cssg_ctx* c = new cssg_ctx();
    c->device = device;
    if (stream) {
        c->stream = (cudaStream_t)stream;
        c->ownStream = false;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete c;
            return cssg_cuda_fail(e, "cudaStreamCreateWithFlags");
        }
        c->ownStream = true;
    }
    *out = c;
    return CSSG_OK;
}

extern "C" int cssg_ctx_destroy(cssg_ctx* c)
{
    if (!c) return CSSG_OK;
    cudaSetDevice(c->device);
    if (c->ownStream) cudaStreamDestroy(c->stream);
    delete c;
    return CSSG_OK;
}

extern "C" int cssg_ctx_synchronize(cssg_ctx* c)
{
    if (!c) return cssg_bad_args("cssg_ctx_synchronize");
    CSSG_CUDA(cudaStreamSynchronize(c->stream));
    return CSSG_OK;
}

extern "C" void* cssg_ctx_stream(cssg_ctx* c) { return c ? (void*)c->stream : nullptr; }
