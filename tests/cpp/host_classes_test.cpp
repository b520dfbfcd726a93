// Exercises the C++ host classes of curvedSpaceSimGPU.hpp the way reference driver code would use them
// (closedMeshSpace::distance / transportParticleAndVectors, gpuSimulation::performTimestep) and prints the results
// as JSON for tests/test_cpp_host.py to compare against the CPU oracle.
//   usage: host_classes_test <mesh.txt> <particles.txt>
//   mesh.txt: nV nF, then vertices, then faces;  particles.txt: n, then face b0 b1 b2 vx vy vz per line
#include <cstdio>
#include <fstream>
#include <vector>

#include "curvedSpaceSimGPU.hpp"

int main(int argc, char** argv)
{
    if (argc < 3) return 2;
    std::ifstream mf(argv[1]), pf(argv[2]);
    int nV, nF;
    mf >> nV >> nF;
    std::vector<double> V(3 * nV);
    std::vector<int> F(3 * nF);
    for (auto& x : V) mf >> x;
    for (auto& x : F) mf >> x;
    int n;
    pf >> n;
    std::vector<cssg::meshPosition> pos(n);
    std::vector<cssg::vector3> vel(n);
    for (int i = 0; i < n; ++i) {
        pf >> pos[i].faceIndex >> pos[i].x[0] >> pos[i].x[1] >> pos[i].x[2] >> vel[i][0] >> vel[i][1] >> vel[i][2];
    }
    cssg::closedMeshSpace space;
    space.loadMesh(V, F);
    // distances from particle 0 to all others (whole mesh)
    std::vector<cssg::meshPosition> targets(pos.begin() + 1, pos.end());
    std::vector<double> d;
    std::vector<cssg::vector3> ts, te;
    space.distance(pos[0], targets, d, ts, te);
    // walk particle 1 by its velocity, transporting the velocity
    cssg::meshPosition p1 = pos[1];
    cssg::vector3 disp = vel[1];
    std::vector<cssg::vector3> tv{vel[1]};
    space.transportParticleAndVectors(p1, disp, tv);
    // 10 NVE steps of the whole system, sigma = 0.3, all-to-all
    cssg::harmonicRepulsion force(1.0 / 0.09, 0.3);
    cssg::gpuSimulation sim(space, n, force, cssg::gpuSimulation::NVE, 0.005, 0.0, 1.0, 2, false);
    sim.positions = pos;
    sim.velocities = vel;
    sim.push();
    sim.performTimestep(10);
    sim.pull();
    // the same 10 steps with the state kept in the public vectors (one library call)
    cssg::gpuSimulation sim2(space, n, force, cssg::gpuSimulation::NVE, 0.005, 0.0, 1.0, 2, false);
    sim2.positions = pos;
    sim2.velocities = vel;
    sim2.performTimestepFromHost(10);
    // simpleModel::findNeighbors at the initial positions: neighbour lists from the device's pair records
    cssg::gpuSimulation sim3(space, n, force, cssg::gpuSimulation::NVE, 0.005, 0.0, 1.0, 2, false);
    sim3.positions = pos;
    sim3.velocities = vel;
    sim3.push();
    sim3.findNeighbors();
    printf("{\"area\": %.17g, \"d\": [", space.getArea());
    for (size_t i = 0; i < d.size(); ++i) printf("%s%.17g", i ? ", " : "", d[i]);
    printf("], \"ts\": [");
    for (size_t i = 0; i < ts.size(); ++i) printf("%s%.17g, %.17g, %.17g", i ? ", " : "", ts[i][0], ts[i][1], ts[i][2]);
    printf("], \"walk\": [%d, %.17g, %.17g, %.17g, %.17g, %.17g, %.17g]", p1.faceIndex, p1.x[0], p1.x[1], p1.x[2],
           tv[0][0], tv[0][1], tv[0][2]);
    printf(", \"face\": [");
    for (int i = 0; i < n; ++i) printf("%s%d", i ? ", " : "", sim.positions[i].faceIndex);
    printf("], \"bary\": [");
    for (int i = 0; i < n; ++i)
        printf("%s%.17g, %.17g, %.17g", i ? ", " : "", sim.positions[i].x[0], sim.positions[i].x[1], sim.positions[i].x[2]);
    printf("], \"face2\": [");
    for (int i = 0; i < n; ++i) printf("%s%d", i ? ", " : "", sim2.positions[i].faceIndex);
    printf("], \"bary2\": [");
    for (int i = 0; i < n; ++i)
        printf("%s%.17g, %.17g, %.17g", i ? ", " : "", sim2.positions[i].x[0], sim2.positions[i].x[1],
               sim2.positions[i].x[2]);
    printf("], \"nb0\": [");
    for (size_t k = 0; k < sim3.neighbors[0].size(); ++k) printf("%s%d", k ? ", " : "", sim3.neighbors[0][k]);
    printf("], \"nd0\": [");  // -1 for +inf (beyond the cutoff)
    for (size_t k = 0; k < sim3.neighborDistances[0].size(); ++k) {
        const double x = sim3.neighborDistances[0][k];
        printf("%s%.17g", k ? ", " : "", std::isinf(x) ? -1.0 : x);
    }
    printf("]}\n");
    return 0;
}
