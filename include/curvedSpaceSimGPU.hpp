// curvedSpaceSimGPU.hpp - C++ host classes over the C ABI (cssg.h) that keep the reference's interfaces for the
// per-timestep hot path, so existing curvedSpaceSim driver code can switch to the GB300 kernels with type changes
// only.  Header-only; link against libcssg.so and the CUDA runtime.
//
//   reference                                   here
//   meshPosition (inc/pointDataType.h:10-28)    cssg::meshPosition     (x = barycentric weights, faceIndex)
//   closedMeshSpace / triangulatedMeshSpace     cssg::closedMeshSpace
//     distance (triangulatedMeshSpace.cpp:212-238, distanceWithSubmeshing :155-205)
//     transportParticleAndVectors (:448-564), displaceParticle (:428-432), getArea (:153),
//     useSubmeshingRoutines (triangulatedMeshSpace.h:60-66), randomPosition (:108-116),
//     randomVectorAtPosition (:118-138)
//   simpleModel (src/models/simpleModel.h:25-111) + force + updater + simulation
//                                               cssg::gpuSimulation: positions/velocities/forces vectors,
//                                               moveParticles, computeForces, performTimestep on the device
//   harmonicRepulsion (src/forces/harmonicRepulsion.cpp:3-34)
//                                               cssg::harmonicRepulsion::pairwiseForce / pairwiseEnergy
//
// Errors: the reference prints and throws std::exception (inc/debuggingHelp.h:19-31); these classes throw
// std::runtime_error carrying cssg_last_error() or the per-item status name.
#ifndef CURVEDSPACESIM_GPU_HPP
#define CURVEDSPACESIM_GPU_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <fstream>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "cssg.h"
#include "curvedSpaceSimDatabase.hpp"

namespace cssg {

struct vector3 {
    double v[3] = {0, 0, 0};
    vector3() = default;
    vector3(double a, double b, double c) : v{a, b, c} {}
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
    double squared_length() const { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
};
typedef vector3 point3;

struct meshPosition {
    point3 x;  // barycentric weights on faceIndex
    int faceIndex = -1;
    meshPosition() = default;
    meshPosition(point3 b, int f) : x(b), faceIndex(f) {}
};

inline void throwIf(int rc, const char* what)
{
    if (rc != CSSG_OK) throw std::runtime_error(std::string(what) + ": " + cssg_last_error());
}

inline const char* statusName(int st)
{
    switch (st) {
        case CSSG_ST_BORDER: return "Surface is meant to be closed, but a border was encountered.";
        case CSSG_ST_NAN: return "Illegal coordinates";
        case CSSG_ST_VERTEX: return "throughvertex didn't find a face";
        case CSSG_ST_ITER: return "walk exceeded its crossing cap";
        case CSSG_ST_NO_INTERSECTION: return "a barycentric coordinate of the target is negative, but neither 1 nor 2 intersections were found";
        case CSSG_ST_CAPACITY: return "geodesic propagation exceeded its table capacity";
        default: return "ok";
    }
}

// RAII device buffer
template <typename T>
struct devbuf {
    T* p = nullptr;
    size_t n = 0;
    explicit devbuf(size_t count) : n(count)
    {
        if (cudaMalloc((void**)&p, sizeof(T) * (count ? count : 1)) != cudaSuccess) throw std::runtime_error("cudaMalloc");
    }
    ~devbuf() { cudaFree(p); }
    devbuf(const devbuf&) = delete;
    devbuf& operator=(const devbuf&) = delete;
    void up(const T* h, cudaStream_t s)
    {
        if (n) cudaMemcpyAsync(p, h, sizeof(T) * n, cudaMemcpyHostToDevice, s);
    }
    void down(T* h, cudaStream_t s) const
    {
        if (n) cudaMemcpyAsync(h, p, sizeof(T) * n, cudaMemcpyDeviceToHost, s);
    }
};

//! triangulatedMeshSpace::randomPosition (triangulatedMeshSpace.cpp:108-116): a face drawn uniformly by index and
//! weights (u, v, 1 - u - v) with u ~ U(0, 1), v ~ U(0, 1 - u) - not area-uniform, as in the reference.  Host-side
//! initialisation; `nFaces` is the mesh's face count.
template <class Engine>
inline void randomPosition(int nFaces, meshPosition& p, Engine& rng)
{
    std::uniform_real_distribution<double> unit(0.0, 1.0);
    const double x = unit(rng);
    const double y = std::uniform_real_distribution<double>(0.0, 1.0 - x)(rng);
    p.x = point3(x, y, 1.0 - x - y);
    p.faceIndex = std::uniform_int_distribution<int>(0, nFaces - 1)(rng);
}

//! triangulatedMeshSpace::randomVectorAtPosition (triangulatedMeshSpace.cpp:118-138): a Gaussian combination of two
//! orthonormal tangent vectors of the face (the face normal's fixed orthogonaliser and normal x orthogonaliser).
//! V: 3 doubles per vertex; F: 3 vertex indices per face.
template <class Engine>
inline void randomVectorAtPosition(const std::vector<double>& V, const std::vector<int>& F, const meshPosition& p,
                                   vector3& v, Engine& rng)
{
    const double* a = &V[3 * (size_t)F[3 * (size_t)p.faceIndex]];
    const double* b = &V[3 * (size_t)F[3 * (size_t)p.faceIndex + 1]];
    const double* c = &V[3 * (size_t)F[3 * (size_t)p.faceIndex + 2]];
    const double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double nl = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (double& x : n) x /= nl;
    double o[3];
    if (n[0] == 0 && n[1] == 0) {
        o[0] = n[1] - n[2];
        o[1] = n[2] - n[0];
        o[2] = n[0] - n[1];
    } else {
        o[0] = n[1];
        o[1] = -n[0];
        o[2] = 0;
    }
    const double ol = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
    for (double& x : o) x /= ol;
    const double t2[3] = {n[1] * o[2] - n[2] * o[1], n[2] * o[0] - n[0] * o[2], n[0] * o[1] - n[1] * o[0]};
    std::normal_distribution<double> gauss(0.0, 1.0);
    const double g1 = gauss(rng), g2 = gauss(rng);
    v = vector3(g1 * o[0] + g2 * t2[0], g1 * o[1] + g2 * t2[1], g1 * o[2] + g2 * t2[2]);
}

//! closedMeshSpace: a closed triangulated surface whose geodesic work runs on the GPU.
class closedMeshSpace {
public:
    explicit closedMeshSpace(int device = 0) : device_(device) { throwIf(cssg_ctx_create(device, nullptr, &ctx_), "cssg_ctx_create"); }
    virtual ~closedMeshSpace()
    {
        if (mesh_) cssg_mesh_destroy(mesh_);
        cssg_ctx_destroy(ctx_);
    }
    closedMeshSpace(const closedMeshSpace&) = delete;
    closedMeshSpace& operator=(const closedMeshSpace&) = delete;

    //! vertices (x,y,z per vertex) and counter-clockwise triangles
    virtual void loadMesh(const std::vector<double>& V, const std::vector<int>& F)
    {
        if (mesh_) cssg_mesh_destroy(mesh_);
        mesh_ = nullptr;
        throwIf(cssg_mesh_create(V.data(), (int)(V.size() / 3), F.data(), (int)(F.size() / 3), device_, &mesh_),
                "cssg_mesh_create");
        V_ = V;
        F_ = F;
        double bb[6];
        throwIf(cssg_mesh_info(mesh_, nullptr, nullptr, &area_, bb), "cssg_mesh_info");
        for (int c = 0; c < 3; ++c) {
            minVertexPosition[c] = bb[c];
            maxVertexPosition[c] = bb[3 + c];
        }
    }

    //! OFF reader (the reference loads OFF/OBJ/STL/PLY through CGAL; triangles only, like its is_triangle_mesh check)
    void loadMeshFromFile(const std::string& filename, bool verbose = false)
    {
        std::ifstream in(filename);
        if (!in) throw std::runtime_error("Invalid input file.");
        std::string tok;
        std::vector<std::string> toks;
        std::string line;
        while (std::getline(in, line)) {
            auto h = line.find('#');
            if (h != std::string::npos) line = line.substr(0, h);
            std::istringstream ss(line);
            while (ss >> tok) toks.push_back(tok);
        }
        size_t p = 0;
        if (!toks.empty() && (toks[0] == "OFF" || toks[0] == "off")) p = 1;
        int nv = std::stoi(toks.at(p)), nf = std::stoi(toks.at(p + 1));
        p += 3;
        std::vector<double> V(3 * (size_t)nv);
        for (size_t i = 0; i < V.size(); ++i) V[i] = std::stod(toks.at(p++));
        std::vector<int> F;
        F.reserve(3 * (size_t)nf);
        for (int f = 0; f < nf; ++f) {
            int k = std::stoi(toks.at(p++));
            if (k != 3) throw std::runtime_error("Non-triangular mesh");
            for (int c = 0; c < 3; ++c) F.push_back(std::stoi(toks.at(p++)));
        }
        if (verbose) printf("input mesh has %i faces and %i vertices\n", nf, nv);
        loadMesh(V, F);
    }

    void useSubmeshingRoutines(bool useSubMesh, double maxDist = 1.0, bool danger = false)
    {
        submeshingActivated_ = useSubMesh;
        maximumDistance_ = maxDist;
        (void)danger;
    }

    double getArea() const { return area_; }

    //! geodesic distances and unit path tangents from p1 to every p2 (the reference's per-source query)
    void distance(meshPosition& p1, std::vector<meshPosition>& p2, std::vector<double>& distances,
                  std::vector<vector3>& startPathTangent, std::vector<vector3>& endPathTangent,
                  double distanceThreshold = 1e20)
    {
        const int n = (int)p2.size();
        distances.resize(n);
        startPathTangent.resize(n);
        endPathTangent.resize(n);
        if (n == 0) return;
        cudaStream_t s = (cudaStream_t)cssg_ctx_stream(ctx_);
        std::vector<int> sf{p1.faceIndex}, off{0, n}, cf(n);
        std::vector<double> sb{p1.x[0], p1.x[1], p1.x[2]}, cb(3 * (size_t)n), th{distanceThreshold};
        for (int i = 0; i < n; ++i) {
            cf[i] = p2[i].faceIndex;
            for (int c = 0; c < 3; ++c) cb[3 * i + c] = p2[i].x[c];
        }
        devbuf<int> dsf(1), doff(2), dcf(n), dst(1);
        devbuf<double> dsb(3), dcb(3 * (size_t)n), dth(1), dd(n), dts(3 * (size_t)n), dte(3 * (size_t)n);
        dsf.up(sf.data(), s);
        doff.up(off.data(), s);
        dcf.up(cf.data(), s);
        dsb.up(sb.data(), s);
        dcb.up(cb.data(), s);
        dth.up(th.data(), s);
        throwIf(cssg_distance_batch(ctx_, mesh_, 1, dsf.p, dsb.p, doff.p, dcf.p, dcb.p, submeshingActivated_ ? 1 : 0,
                                    maximumDistance_, dth.p, INFINITY, dd.p, dts.p, dte.p, dst.p, nullptr),
                "cssg_distance_batch");
        std::vector<double> ts(3 * (size_t)n), te(3 * (size_t)n);
        int st = 0;
        dd.down(distances.data(), s);
        dts.down(ts.data(), s);
        dte.down(te.data(), s);
        dst.down(&st, s);
        throwIf(cssg_ctx_synchronize(ctx_), "cssg_ctx_synchronize");
        if (st) throw std::runtime_error(statusName(st));
        for (int i = 0; i < n; ++i) {
            startPathTangent[i] = vector3(ts[3 * i], ts[3 * i + 1], ts[3 * i + 2]);
            endPathTangent[i] = vector3(te[3 * i], te[3 * i + 1], te[3 * i + 2]);
        }
    }

    //! move pos by displacementVector along the surface, parallel-transporting transportVectors
    void transportParticleAndVectors(meshPosition& pos, vector3& displacementVector, std::vector<vector3>& transportVectors)
    {
        std::vector<meshPosition> p{pos};
        std::vector<vector3> d{displacementVector};
        std::vector<std::vector<vector3>> t{transportVectors};
        transportBatch(p, d, t);
        pos = p[0];
        displacementVector = d[0];
        transportVectors = t[0];
    }

    void displaceParticle(meshPosition& pos, vector3& displacementVector)
    {
        std::vector<vector3> none;
        transportParticleAndVectors(pos, displacementVector, none);
    }

    //! batched walk (what simpleModel::moveParticles does particle by particle)
    void transportBatch(std::vector<meshPosition>& pos, std::vector<vector3>& disp,
                        std::vector<std::vector<vector3>>& transport)
    {
        const int n = (int)pos.size();
        if (n == 0) return;
        const int nt = transport.empty() ? 0 : (int)transport[0].size();
        cudaStream_t s = (cudaStream_t)cssg_ctx_stream(ctx_);
        std::vector<int> f(n), st(n);
        std::vector<double> b(3 * (size_t)n), d(3 * (size_t)n), tv(3 * (size_t)n * nt);
        for (int i = 0; i < n; ++i) {
            f[i] = pos[i].faceIndex;
            for (int c = 0; c < 3; ++c) {
                b[3 * i + c] = pos[i].x[c];
                d[3 * i + c] = disp[i][c];
            }
            for (int k = 0; k < nt; ++k)
                for (int c = 0; c < 3; ++c) tv[3 * ((size_t)i * nt + k) + c] = transport[i][k][c];
        }
        devbuf<int> df(n), dst(n);
        devbuf<double> db(3 * (size_t)n), dd(3 * (size_t)n), dtv(3 * (size_t)n * nt);
        df.up(f.data(), s);
        db.up(b.data(), s);
        dd.up(d.data(), s);
        dtv.up(tv.data(), s);
        throwIf(cssg_transport_batch(ctx_, mesh_, n, df.p, db.p, dd.p, nt ? dtv.p : nullptr, nt, dst.p, nullptr),
                "cssg_transport_batch");
        df.down(f.data(), s);
        db.down(b.data(), s);
        dd.down(d.data(), s);
        dtv.down(tv.data(), s);
        dst.down(st.data(), s);
        throwIf(cssg_ctx_synchronize(ctx_), "cssg_ctx_synchronize");
        for (int i = 0; i < n; ++i) {
            if (st[i]) throw std::runtime_error(statusName(st[i]));
            pos[i].faceIndex = f[i];
            pos[i].x = point3(b[3 * i], b[3 * i + 1], b[3 * i + 2]);
            disp[i] = vector3(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
            for (int k = 0; k < nt; ++k)
                transport[i][k] = vector3(tv[3 * ((size_t)i * nt + k)], tv[3 * ((size_t)i * nt + k) + 1],
                                          tv[3 * ((size_t)i * nt + k) + 2]);
        }
    }

    //! triangulatedMeshSpace::meshPositionToEuclideanLocation: R3 points of mesh positions (PMP::construct_point)
    void meshPositionToEuclideanLocation(const std::vector<meshPosition>& p, std::vector<double>& out) const
    {
        out.resize(3 * p.size());
        for (size_t i = 0; i < p.size(); ++i) {
            const int* f = &F_[3 * (size_t)p[i].faceIndex];
            const double s = p[i].x[0] + p[i].x[1] + p[i].x[2];
            for (int c = 0; c < 3; ++c)
                out[3 * i + c] = (p[i].x[0] * V_[3 * (size_t)f[0] + c] + p[i].x[1] * V_[3 * (size_t)f[1] + c] +
                                  p[i].x[2] * V_[3 * (size_t)f[2] + c]) / s;
        }
    }

    //! triangulatedMeshSpace::randomPosition / randomVectorAtPosition on this mesh (host-side initialisation)
    template <class Engine>
    void randomPosition(meshPosition& p, Engine& rng) const
    {
        cssg::randomPosition((int)(F_.size() / 3), p, rng);
    }
    template <class Engine>
    void randomVectorAtPosition(meshPosition& p, vector3& v, Engine& rng) const
    {
        cssg::randomVectorAtPosition(V_, F_, p, v, rng);
    }

    cssg_ctx* context() const { return ctx_; }
    cssg_mesh* mesh() const { return mesh_; }
    bool submeshing() const { return submeshingActivated_; }
    double maximumDistance() const { return maximumDistance_; }

    double minVertexPosition[3] = {0, 0, 0};
    double maxVertexPosition[3] = {0, 0, 0};

private:
    int device_;
    cssg_ctx* ctx_ = nullptr;
    cssg_mesh* mesh_ = nullptr;
    std::vector<double> V_;
    std::vector<int> F_;
    double area_ = 0;
    bool submeshingActivated_ = false;
    double maximumDistance_ = 0;
};

//! openMeshSpace with tangential walls (tangentialOpenMeshSpace.cpp): walks slide along the border and transported
//! vectors that point out of the surface are projected onto the wall.
class tangentialOpenMeshSpace : public closedMeshSpace {
public:
    explicit tangentialOpenMeshSpace(int device = 0) : closedMeshSpace(device) {}
    void loadMesh(const std::vector<double>& V, const std::vector<int>& F) override
    {
        closedMeshSpace::loadMesh(V, F);
        throwIf(cssg_mesh_set_boundary(mesh(), 1), "cssg_mesh_set_boundary");
    }
};

//! openMeshSpace with absorbing walls (absorbingOpenMeshSpace.cpp): a walk that reaches the border stops there.
class absorbingOpenMeshSpace : public closedMeshSpace {
public:
    explicit absorbingOpenMeshSpace(int device = 0) : closedMeshSpace(device) {}
    void loadMesh(const std::vector<double>& V, const std::vector<int>& F) override
    {
        closedMeshSpace::loadMesh(V, F);
        throwIf(cssg_mesh_set_boundary(mesh(), 2), "cssg_mesh_set_boundary");
    }
};

//! harmonicRepulsion: E = k/2 (sigma - d)^2 for d < sigma, F = -k (sigma - d) t for d <= sigma
class harmonicRepulsion {
public:
    harmonicRepulsion(double stiffness = 1, double monodisperseRange = 1) : k(stiffness), sigma(monodisperseRange),
        maximumInteractionRange(monodisperseRange) {}
    double pairwiseEnergy(const vector3&, double distance) const
    {
        return distance < sigma ? 0.5 * k * (sigma - distance) * (sigma - distance) : 0.0;
    }
    vector3 pairwiseForce(const vector3& separation, double distance) const
    {
        if (distance > sigma) return vector3();
        double m = -k * (sigma - distance);
        return vector3(m * separation[0], m * separation[1], m * separation[2]);
    }
    double k, sigma, maximumInteractionRange;
};

//! simpleModel's neighbour lists (simpleModel.h:75-79, filled by findNeighbors, simpleModel.cpp:68-112) from the
//! pair records of cssg_system_pairs (grouped by source): per particle the candidate indices, the unit start tangents
//! (neighborVectors) and the geodesic distances.  Distances beyond the force cutoff are +inf (the device does not
//! resolve them further); pairs the learned screen skipped (j < 0, index -j - 1) carry their index and +inf.
inline void pairsToNeighborLists(int N, int count, const int* i, const int* j, const double* d, const double* t,
                                 std::vector<std::vector<int>>& neighbors,
                                 std::vector<std::vector<vector3>>& neighborVectors,
                                 std::vector<std::vector<double>>& neighborDistances)
{
    neighbors.assign(N, {});
    neighborVectors.assign(N, {});
    neighborDistances.assign(N, {});
    for (int k = 0; k < count; ++k) {
        const int a = i[k];
        if (a < 0 || a >= N) continue;
        const bool screened = j[k] < 0;
        neighbors[a].push_back(screened ? -j[k] - 1 : j[k]);
        neighborVectors[a].push_back(vector3(t[3 * (size_t)k], t[3 * (size_t)k + 1], t[3 * (size_t)k + 2]));
        neighborDistances[a].push_back(screened ? HUGE_VAL : d[k]);
    }
}

//! simpleModel + harmonicRepulsion + (velocityVerletNVE | noseHooverNVT) + simulation, resident on the GPU.
//! performTimestep() advances one step without leaving the device; positions/velocities/forces are mirrored into
//! the public vectors by pull() and pushed by push(), like the reference model's public members.
class gpuSimulation {
public:
    enum Integrator { NVE = 0, NVT = 1 };
    gpuSimulation(closedMeshSpace& space, int N, const harmonicRepulsion& force, Integrator integ, double dt,
                  double T = 0.0, double tau = 1.0, int chainLength = 2, bool useCellList = true)
        : space_(space), N(N)
    {
        cssg_params p{};
        p.integrator = integ;
        p.force_kind = 0;
        p.k = force.k;
        p.sigma = force.sigma;
        p.range = useCellList ? force.maximumInteractionRange : 0.0;
        p.submesh = space.submeshing() ? 1 : 0;
        p.max_dist = space.submeshing() ? space.maximumDistance() : force.sigma;
        p.cutoff = force.sigma;
        p.dt = dt;
        p.temperature = T;
        p.tau = tau;
        p.chain_length = chainLength;
        throwIf(cssg_system_create(space.context(), space.mesh(), N, &p, &sys_), "cssg_system_create");
        positions.resize(N);
        velocities.resize(N);
        forces.resize(N);
    }
    ~gpuSimulation() { cssg_system_destroy(sys_); }
    gpuSimulation(const gpuSimulation&) = delete;
    gpuSimulation& operator=(const gpuSimulation&) = delete;

    void setParticlePositions(const std::vector<meshPosition>& p)
    {
        positions = p;
        push();
    }
    void push()
    {
        std::vector<int> f(N);
        std::vector<double> b(3 * (size_t)N), v(3 * (size_t)N), fo(3 * (size_t)N);
        for (int i = 0; i < N; ++i) {
            f[i] = positions[i].faceIndex;
            for (int c = 0; c < 3; ++c) {
                b[3 * i + c] = positions[i].x[c];
                v[3 * i + c] = velocities[i][c];
                fo[3 * i + c] = forces[i][c];
            }
        }
        throwIf(cssg_system_set_state(sys_, f.data(), b.data(), v.data(), fo.data()), "cssg_system_set_state");
    }
    void pull()
    {
        std::vector<int> f(N);
        std::vector<double> b(3 * (size_t)N), v(3 * (size_t)N), fo(3 * (size_t)N);
        throwIf(cssg_system_get_state(sys_, f.data(), b.data(), v.data(), fo.data()), "cssg_system_get_state");
        for (int i = 0; i < N; ++i) {
            positions[i] = meshPosition(point3(b[3 * i], b[3 * i + 1], b[3 * i + 2]), f[i]);
            velocities[i] = vector3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
            forces[i] = vector3(fo[3 * i], fo[3 * i + 1], fo[3 * i + 2]);
        }
    }
    //! simulation::performTimestep, `steps` times, on the device (CUDA graph replay)
    void performTimestep(int steps = 1)
    {
        throwIf(cssg_system_step(sys_, steps, 1), "cssg_system_step");
        checkItems();
    }
    //! simulation::performTimestep, `steps` times, for a caller that keeps the state in the public vectors: pushes
    //! them, steps on the device and pulls them back in one library call (one synchronisation)
    void performTimestepFromHost(int steps = 1)
    {
        std::vector<int> f(N);
        std::vector<double> b(3 * (size_t)N), v(3 * (size_t)N), fo(3 * (size_t)N);
        for (int i = 0; i < N; ++i) {
            f[i] = positions[i].faceIndex;
            for (int c = 0; c < 3; ++c) {
                b[3 * i + c] = positions[i].x[c];
                v[3 * i + c] = velocities[i][c];
                fo[3 * i + c] = forces[i][c];
            }
        }
        throwIf(cssg_system_step_host(sys_, steps, f.data(), b.data(), v.data(), fo.data(), f.data(), b.data(),
                                      v.data(), fo.data()),
                "cssg_system_step_host");
        for (int i = 0; i < N; ++i) {
            positions[i] = meshPosition(point3(b[3 * i], b[3 * i + 1], b[3 * i + 2]), f[i]);
            velocities[i] = vector3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
            forces[i] = vector3(fo[3 * i], fo[3 * i + 1], fo[3 * i + 2]);
        }
        checkItems();
    }
    //! gradientDescent::performUpdate (gradientDescent.cpp:6-18), `steps` times: forces, then every particle moved by
    //! deltaT * force; the velocities are carried along when transportVelocities (the model's transport flag)
    void gradientDescent(double deltaT, int steps = 1, bool transportVelocities = false)
    {
        throwIf(cssg_system_gradient_descent(sys_, steps, deltaT, transportVelocities ? 1 : 0),
                "cssg_system_gradient_descent");
        checkItems();
    }
    //! simulation::computeForces
    void computeForces()
    {
        throwIf(cssg_system_compute_forces(sys_), "cssg_system_compute_forces");
        checkItems();
    }
    void checkItems()
    {
        int bits = 0;
        throwIf(cssg_system_check(sys_, &bits, nullptr), "cssg_system_check");
        for (int st = 1; st < 8; ++st)
            if (bits & (1 << st)) throw std::runtime_error(statusName(st));
    }
    cssg_system* handle() const { return sys_; }

    //! fireMinimization::minimizeByFire on the device (fireMinimization.cpp:3-21); parameters as setFIREParameters
    //! (:79-96), the initial deltaT is the simulation's dt.  Returns the iterations used; pulls the state.
    int minimizeByFire(int maximumIterations = 1000, double alphaStart = 0.99, double deltaTMax = 0.1,
                       double deltaTMin = 1e-5, double deltaTInc = 1.1, double deltaTDec = 0.95, double alphaDec = 0.9,
                       int nMin = 4, double forceCutoff = 1e-12, double alphaMin = 0.0, bool reset = false)
    {
        cssg_fire_params fp{maximumIterations, alphaStart, deltaTMax, deltaTMin, deltaTInc, deltaTDec, alphaDec,
                            nMin, forceCutoff, alphaMin};
        double out[5];
        throwIf(cssg_system_fire(sys_, &fp, reset ? 1 : 0, out), "cssg_system_fire");
        checkItems();
        pull();
        forceMax = out[1];
        return (int)out[0];
    }
    //! simulation::computeMonodisperseStress (simulation.cpp:104-173): stress[9], row-major
    void computeMonodisperseStress(std::vector<double>& stress)
    {
        stress.resize(9);
        throwIf(cssg_system_stress(sys_, stress.data()), "cssg_system_stress");
    }
    //! the library's autotuner (band width, CTA size, medium-pass slots, warp cap, source order) on this state
    void autotune(int reps = 2) { throwIf(cssg_system_autotune(sys_, reps, nullptr), "cssg_system_autotune"); }

    //! simpleModel::findNeighbors (simpleModel.cpp:68-112) for host-side analysis: evaluates the forces at the current
    //! device state (candidates, patches, geodesics) and fills neighbors / neighborVectors / neighborDistances from
    //! the pair records (see pairsToNeighborLists).  The first call switches pair recording on for this system.
    void findNeighbors()
    {
        int count = 0;
        if (!pairsEnabled_) {
            throwIf(cssg_system_pairs(sys_, 0, nullptr, nullptr, nullptr, nullptr, &count), "cssg_system_pairs");
            pairsEnabled_ = true;
        }
        computeForces();
        throwIf(cssg_system_pairs(sys_, 0, nullptr, nullptr, nullptr, nullptr, &count), "cssg_system_pairs");
        std::vector<int> i(count), j(count);
        std::vector<double> d(count), t(3 * (size_t)count);
        throwIf(cssg_system_pairs(sys_, count, i.data(), j.data(), d.data(), t.data(), &count), "cssg_system_pairs");
        pairsToNeighborLists(N, count, i.data(), j.data(), d.data(), t.data(), neighbors, neighborVectors,
                             neighborDistances);
    }

    double forceMax = 0;
    closedMeshSpace& space_;
    int N;
    std::vector<meshPosition> positions;
    std::vector<vector3> velocities;
    std::vector<vector3> forces;
    std::vector<std::vector<int>> neighbors;
    std::vector<std::vector<vector3>> neighborVectors;
    std::vector<std::vector<double>> neighborDistances;

private:
    cssg_system* sys_ = nullptr;
    bool pairsEnabled_ = false;
};

//! simpleModelDatabase::writeState for a device-resident simulation: pulls the state and appends a record
inline void writeState(simpleModelDatabase& db, gpuSimulation& sim, double time)
{
    sim.pull();
    const int n = sim.N;
    std::vector<double> r3, bary(3 * (size_t)n), vel(3 * (size_t)n), frc(3 * (size_t)n);
    std::vector<int> face(n), types(n, 0);
    sim.space_.meshPositionToEuclideanLocation(sim.positions, r3);
    for (int i = 0; i < n; ++i) {
        face[i] = sim.positions[i].faceIndex;
        for (int c = 0; c < 3; ++c) {
            bary[3 * i + c] = sim.positions[i].x[c];
            vel[3 * i + c] = sim.velocities[i][c];
            frc[3 * i + c] = sim.forces[i][c];
        }
    }
    db.writeState(r3, bary, face, vel, frc, types, time);
}

//! simpleModelDatabase::readState into a device-resident simulation (fields the database lacks are left unchanged)
inline double readState(const simpleModelDatabase& db, gpuSimulation& sim, int rec)
{
    sim.pull();
    std::vector<double> bary, vel, frc;
    std::vector<int> face, types;
    const double t = db.readState(rec, bary, face, vel, frc, types);
    for (int i = 0; i < sim.N; ++i) {
        sim.positions[i] = meshPosition(point3(bary[3 * i], bary[3 * i + 1], bary[3 * i + 2]), face[i]);
        if (!vel.empty()) sim.velocities[i] = vector3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        if (!frc.empty()) sim.forces[i] = vector3(frc[3 * i], frc[3 * i + 1], frc[3 * i + 2]);
    }
    sim.push();
    return t;
}

}  // namespace cssg

#endif
