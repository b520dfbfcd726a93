/* cssg.h - C ABI of the GB300 (sm_103a) curvedSpaceSim hot path.
 *
 * One shared library (curvedspacesim_gb300/_build/libcssg.so) exports these entry points.  All arguments are
 * plain pointers and sizes; nothing crosses the ABI but C types.  Every function returns an int status
 * (CSSG_OK = 0); per-item errors (a walk that hit a border, a propagation that ran out of queue capacity) are
 * reported in caller-provided int arrays with the CSSG_ST_* codes below, never by exceptions.
 *
 * Pointers are DEVICE pointers unless the name ends in _host.  A context owns a CUDA stream; every launch goes to
 * that stream and returns without synchronising unless the comment says otherwise.
 *
 * Reference interfaces each entry point replaces are cited as path:line in sussmanLab/curvedSpaceSim.
 */
#ifndef CSSG_H
#define CSSG_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ---------------------------------------------------------------------------------------- */
#define CSSG_OK 0
#define CSSG_ERR_ARG 1       /* bad argument (null pointer, negative size, non-triangle mesh) */
#define CSSG_ERR_CUDA 2      /* a CUDA runtime call failed; cssg_last_error() has the message */
#define CSSG_ERR_ITEMS 3     /* at least one item reported a non-zero per-item status */
#define CSSG_ERR_CAPACITY 4  /* a fixed-size buffer was too small (see the function) */

/* ---- per-item status codes (walk and propagation) ------------------------------------------------------------ */
#define CSSG_ST_OK 0
#define CSSG_ST_BORDER 1           /* walk reached a border of a closed-mesh space (triangulatedMeshSpace.cpp:522-548) */
#define CSSG_ST_NAN 2              /* barycentric NaN (meshUtilities.cpp:184-195) */
#define CSSG_ST_VERTEX 3           /* throughVertex found no outgoing face (triangulatedMeshSpace.cpp:339-405) */
#define CSSG_ST_ITER 4             /* walk exceeded its crossing cap */
#define CSSG_ST_NO_INTERSECTION 5  /* target outside the face but no edge crossing found (:534-541) */
#define CSSG_ST_CAPACITY 6         /* propagation queue / table capacity exceeded for this source */

typedef struct cssg_mesh cssg_mesh;     /* device-resident mesh with connectivity and edge frames */
typedef struct cssg_ctx cssg_ctx;       /* stream + scratch for batched calls; use one per host thread */
typedef struct cssg_system cssg_system; /* device-resident particle system (model + force + updater state) */

/* Message of the last error on this thread (static storage). */
const char* cssg_last_error(void);
/* Library version string. */
const char* cssg_version(void);

/* ---- mesh ------------------------------------------------------------------------------------------------------
 * Replaces triangulatedMeshSpace::loadMeshFromFile + updateMeshSpanAndTree (src/models/triangulatedMeshSpace.cpp:6-72):
 * host arrays vertices_host[3*nV] (x,y,z) and faces_host[3*nF] (counter-clockwise vertex indices; the order also
 * defines the barycentric order of positions on that face).  Builds adjacency, edge frames, vertex rings, angle
 * sums and the bounding box on the host and uploads them. */
int cssg_mesh_create(const double* vertices_host, int nV, const int* faces_host, int nF, int device, cssg_mesh** out);
/* Releases the mesh (the reference's triangulatedMeshSpace destructor). */
int cssg_mesh_destroy(cssg_mesh* mesh);
/* area (triangulatedMeshSpace::getArea, :153), bbox_host[6] = min xyz, max xyz with the origin included (:6-30). */
int cssg_mesh_info(const cssg_mesh* mesh, int* nV, int* nF, double* area, double* bbox_host);

/* Boundary condition of walks on this mesh (the reference picks it by the space class): 0 closed
 * (triangulatedMeshSpace: a border edge or vertex is the per-item error CSSG_ST_BORDER), 1 tangential
 * (tangentialOpenMeshSpace.cpp: slide along the border, transported vectors that point out are projected), 2 absorbing
 * (absorbingOpenMeshSpace.cpp: stop at the border).  Systems copy it when they are created.  At a border vertex the
 * next border heading is the edge of the vertex's other faces that overlaps most with the displacement (the rule
 * stated in openMeshSpace.cpp:35-37); the reference's candidate loop depends on CGAL internals and is not followed. */
int cssg_mesh_set_boundary(cssg_mesh* mesh, int bc);

/* ---- context ----------------------------------------------------------------------------------------------- */
/* No reference counterpart (the reference is single-threaded host code): a device and a stream for batched calls.
 * stream: a cudaStream_t, or NULL to create a private non-blocking stream. */
int cssg_ctx_create(int device, void* stream, cssg_ctx** out);
int cssg_ctx_destroy(cssg_ctx* ctx);
int cssg_ctx_synchronize(cssg_ctx* ctx);
void* cssg_ctx_stream(cssg_ctx* ctx);

/* ---- walk: triangulatedMeshSpace::transportParticleAndVectors, batched ----------------------------------------
 * Replaces src/models/triangulatedMeshSpace.cpp:448-564 (plus :247-407, :566-658) called once per particle by
 * simpleModel::moveParticles (src/models/simpleModel.cpp:44-66).  In place: face[n], bary[3n], disp[3n] (modified
 * the same way the reference modifies its displacementVector), transport[n*nTransport*3] (vectors carried along,
 * e.g. velocities).  status[n] gets CSSG_ST_* per particle; crossings (nullable) accumulates the edge+vertex
 * crossings of the launch in one unsigned long long on the device. */
int cssg_transport_batch(cssg_ctx* ctx, const cssg_mesh* mesh, int n, int* face, double* bary, double* disp,
                         double* transport, int nTransport, int* status, unsigned long long* crossings);

/* ---- distances: triangulatedMeshSpace::distance / distanceWithSubmeshing, batched over sources -----------------
 * Replaces src/models/triangulatedMeshSpace.cpp:155-238 with computePathDistanceAndTangents
 * (src/utility/meshUtilities.cpp:360-380), called once per source by simpleModel::findNeighbors
 * (src/models/simpleModel.cpp:68-112).
 *   sources: src_face[nSrc], src_bary[3*nSrc]
 *   targets: CSR cand_offsets[nSrc+1] into cand_face[], cand_bary[3*]
 *   submesh = 0: whole mesh; submesh = 1: the reference's patch (submesher.cpp:55-147) of radius
 *            min(max_dist, threshold[i]) per source (threshold nullable = +inf)
 *   cutoff: paths longer than cutoff are not followed; such targets report +inf (use +inf for exact reference
 *           semantics, where a disconnected patch target reports 2*max_dist and tangent (0,0,1) (:197-203))
 * Outputs per candidate: d_out[], tstart_out[3*] (unit start tangent at the source), tend_out[3*] (nullable; unit
 * direction of travel at the target).  status[nSrc].  stats (nullable): 4 per source = windows processed,
 * pseudo-source launches, propagation rounds, targets. */
int cssg_distance_batch(cssg_ctx* ctx, const cssg_mesh* mesh, int nSrc, const int* src_face, const double* src_bary,
                        const int* cand_offsets, const int* cand_face, const double* cand_bary, int submesh,
                        double max_dist, const double* threshold, double cutoff, double* d_out, double* tstart_out,
                        double* tend_out, int* status, long long* stats);

/* ---- distances without allocation -----------------------------------------------------------------------------
 * No reference counterpart: the reference allocates freely on the host.  Same arguments, kernels and results as
 * cssg_distance_batch, but it allocates and frees no device memory: its scratch is a fixed, file-scope device
 * buffer of CSSG_NOALLOC_SCRATCH_BYTES (64 MiB) in the library, plus a few words for the work counter, the system
 * descriptor and the largest candidate count.  For host codes that cannot call the allocator during a step.
 *   - A call whose single propagation slot (set by the largest candidate count and the reach, as in
 *     cssg_distance_batch) exceeds the scratch returns CSSG_ERR_CAPACITY and launches nothing; a call that fits
 *     fewer slots than cssg_distance_batch would use runs with fewer slots (same results, less parallelism).
 *   - Each call resets what must start at zero (the work counter) and empties the slots' tables itself.
 *   - The scratch is shared by every call on a device: calls that overlap in time on one device (different
 *     streams or contexts, or several host threads) race on it.  Calls issued on one stream are ordered.
 *   - The first call on each device looks up the scratch's device address (cudaGetSymbolAddress) and must not be
 *     made while a stream is being captured.
 *   - Like cssg_distance_batch it reads the largest candidate count back to the host, so it synchronises the
 *     context's stream once. */
#define CSSG_NOALLOC_SCRATCH_BYTES (64u << 20)
int cssg_distance_batch_noalloc(cssg_ctx* ctx, const cssg_mesh* mesh, int nSrc, const int* src_face,
                                const double* src_bary, const int* cand_offsets, const int* cand_face,
                                const double* cand_bary, int submesh, double max_dist, const double* threshold,
                                double cutoff, double* d_out, double* tstart_out, double* tend_out, int* status,
                                long long* stats);

/* ---- particle system: simpleModel + force + updater on the device -------------------------------------------- */
typedef struct cssg_params {
    int integrator;      /* 0 velocityVerletNVE (velocityVerletNVE.cpp:3-29), 1 noseHooverNVT (noseHooverNVT.cpp:3-150) */
    int force_kind;      /* 0 harmonicRepulsion (harmonicRepulsion.cpp:3-34), 1 gaussianRepulsion (gaussianRepulsion.cpp:3-12) */
    double k;            /* harmonic stiffness / gaussian alpha */
    double sigma;        /* harmonic range / gaussian width */
    double range;        /* candidate range (force maximumInteractionRange); <= 0: all-to-all (baseNeighborStructure) */
    int submesh;         /* 1: per-source reference patches (useSubmeshingRoutines(true, max_dist)) */
    double max_dist;     /* submesh radius cap */
    double cutoff;       /* geodesic pruning radius, >= the largest distance a force reads (sigma for harmonic) */
    double dt;           /* timestep */
    double temperature;  /* NVT target temperature */
    double tau;          /* NVT chain time scale */
    int chain_length;    /* NVT chain length M (default 2) */
} cssg_params;

/* simpleModel(n) + setSpace + setNeighborStructure (src/models/simpleModel.h:29-39), a force (baseForce.h) and an
 * updater (velocityVerletNVE.h / noseHooverNVT.h) bound into one device-resident system; state starts at zero. */
int cssg_system_create(cssg_ctx* ctx, const cssg_mesh* mesh, int n, const cssg_params* params, cssg_system** out);
/* K independent systems (own mesh, particle count and force / patch parameters) advanced together: every kernel of
 * a step serves all of them (one persistent geodesic launch per step over all sources).  Integrator, dt, T, tau,
 * chain length and the neighbour-structure kind (cell list or all-to-all) must agree.  State arrays of the other
 * system_* calls are the concatenation of the systems' particles in order. */
int cssg_system_create_batched(cssg_ctx* ctx, int K, const cssg_mesh* const* meshes, const int* counts,
                               const cssg_params* params, cssg_system** out);
/* Releases the system (no reference counterpart beyond the objects' destructors). */
int cssg_system_destroy(cssg_system* sys);
/* simpleModel::setParticlePositions (simpleModel.cpp:204-212) + velocities/forces; host arrays; nullable fields
 * are left unchanged.  Synchronises. */
int cssg_system_set_state(cssg_system* sys, const int* face_host, const double* bary_host, const double* vel_host,
                          const double* force_host);
/* noseHooverNVT::setBathVariables (noseHooverNVT.cpp:28-36): chain masses from N, T, tau; chain at rest.  Called by
 * cssg_system_create; call again after replacing the particles of an NVT system. */
int cssg_system_reset_thermostat(cssg_system* sys);
/* The model's public state vectors positions / velocities / forces (simpleModel.h:68-72) copied to host arrays
 * (nullable) and synchronises. */
int cssg_system_get_state(cssg_system* sys, int* face_host, double* bary_host, double* vel_host, double* force_host);
/* Device pointers of the state arrays (face[n], bary[3n], vel[3n], force[3n]); no reference counterpart. */
int cssg_system_device_state(cssg_system* sys, int** face, double** bary, double** vel, double** force);
/* simulation::performTimestep x steps (simulation.cpp:84-95); asynchronous on the context stream.  use_graph=1
 * replays one captured CUDA graph per step. */
int cssg_system_step(cssg_system* sys, int steps, int use_graph);
/* simulation::performTimestep x steps (simulation.cpp:84-95) from and to host state, in one call: the state arrays
 * given in *_in (nullable; host memory, pinned for overlap) are copied in, the steps run as graph replays, the state
 * is copied out to *_out (nullable; may alias *_in), then the call synchronises once.  Same checks as
 * cssg_system_set_state.  A caller that keeps its state on the host (the reference's simpleModel owns host vectors)
 * pays one synchronisation per call instead of one per set_state, get_state and step. */
int cssg_system_step_host(cssg_system* sys, int steps, const int* face_in, const double* bary_in, const double* vel_in,
                          const double* force_in, int* face_out, double* bary_out, double* vel_out, double* force_out);
/* simulation::computeForces (simulation.cpp:61-70 -> baseForce.cpp:12-28): neighbours, geodesics, forces. */
int cssg_system_compute_forces(cssg_system* sys);

/* ---- FIRE minimisation: fireMinimization::minimizeByFire (src/updaters/fireMinimization.cpp:3-21) ------------------
 * Replaces the reference's performUpdate of a fireMinimization updater: forces, then until forceMax <= force_cutoff
 * or maximum_iterations: velocity-Verlet half steps (velocityVerletNVE.cpp:14-29) with force and velocity carried by
 * the walk (simpleModel.cpp:44-66), fireStep (fireMinimization.cpp:38-77), getMaxForce (baseUpdater.cpp:39-54).
 * Fields as setFIREParameters (:79-96).  The initial deltaT is the system's dt (the reference's setFIREParameters
 * does not apply its _deltaT argument either).  deltaT, alpha and nSinceNegativePower persist between calls like the
 * reference's members; reset = 1 (or the first call) restarts them at (dt, alpha_start, 0).  A batched object
 * (cssg_system_create_batched) minimises every system at once, each with its own FIRE state and stopping rule (one
 * fireMinimization updater per system, same parameters): a converged system stops moving while the others go on.
 * result_host (nullable, 5 doubles per system) = {iterations, forceMax, deltaT, alpha, nSinceNegativePower} for
 * system 0, then system 1, ...  Synchronises. */
typedef struct cssg_fire_params {
    int maximum_iterations;
    double alpha_start, dt_max, dt_min, dt_inc, dt_dec, alpha_dec;
    int n_min;
    double force_cutoff, alpha_min;
} cssg_fire_params;
int cssg_system_fire(cssg_system* sys, const cssg_fire_params* params, int reset, double* result_host);

/* ---- gradient descent: gradientDescent::performUpdate (src/updaters/gradientDescent.cpp:6-18) x steps --------------
 * Each step computes the forces at the current positions, then moves every particle by deltaT * force with the walk
 * (simpleModel::moveParticles, simpleModel.cpp:44-66).  transport_velocity = 1 carries the velocities along
 * (the model's particleShiftsRequireVelocityTransport, set when an NVE/NVT/FIRE updater was attached before); the
 * reference's gradient-descent updater sets no transport flag itself.  The forces left in the state are the last
 * ones computed (before the last move).  Asynchronous on the context stream; failures via cssg_system_check. */
int cssg_system_gradient_descent(cssg_system* sys, int steps, double delta_t, int transport_velocity);

/* simulation::computeMonodisperseStress (src/simulation/simulation.cpp:104-173): recomputes the neighbour pairs on the
 * current positions and returns stress_host[9] (row-major 3x3) = rho <v (x) v> / (2N) + <f_ij (x) t_ij> / (4 A N),
 * rho = N / A, kB = 1; like the reference, v_i (x) v_i is summed once per neighbour pair of i.  Enables pair output.
 * One system per object; CSSG_ERR_CAPACITY if a source has more candidates than the pair buffer.  Synchronises. */
int cssg_system_stress(cssg_system* sys, double* stress_host);

/* Tuning of the propagation passes (no reference counterpart).  delta_scale: band width of the distance-banded
 * rounds in units of each mesh's mean edge length (default 1); warps_per_block: warps of the persistent launches'
 * blocks (1..8, default 8; the grid always covers every SM equally); mid_slots: source groups of the medium-tier pass
 * (<= the number allocated at creation; <= 0 keeps the current value); warps_per_sm: > 0 caps the source warps of
 * the regular pass per SM (0: all slots); lpt_order: 1 processes sources longest first by their cost in the last
 * force evaluation, 0 in cell order; warps_per_source: 1, 2, 4 or 8 warps solve one source together (a few sources
 * on many SMs want more); wide_registers: the kernel build, bit 0 = up to 255 registers per thread (no register
 * spills, at most 8 warps per SM; else 128), bit 1 = hash-table probes out of line (a smaller kernel, faster where
 * sources are small).  Results do not depend on these, only the work and its balance do.
 * Drops the captured step graph. */
int cssg_system_set_tuning(cssg_system* sys, double delta_scale, int warps_per_block, int mid_slots, int warps_per_sm,
                           int lpt_order, int warps_per_source, int wide_registers);
/* Autotuner: times `reps` force evaluations on the current state for each candidate (delta_scale in {0.5, 1, 2, 4}
 * x (warps_per_block, warps_per_sm, lpt_order, warps_per_source, wide_registers) in {(8,0,0,1,0), (4,0,0,1,0),
 * (8,0,1,1,0), (8,8,1,1,0), (8,4,1,1,0), (8,0,1,2,0), (8,0,1,4,0), (8,0,1,8,0), (8,0,1,1,1), (8,0,1,2,1),
 * (8,0,1,4,1), (8,0,1,1,3), (8,0,1,1,2), (8,0,1,2,3)} x medium slots in {allocated, 8 per SM}), then, on single
 * cell-list systems, the one-source-per-lane pass (cssg_system_set_lanes) with 16 and 32 lanes x lpt_order in {0, 1} x the
 * splits of cssg_system_set_lane_split, then the medium and large passes' group sizes (cssg_system_set_pass_groups);
 * rejects candidates that overflow a table, keeps the fastest (a lane-pass candidate only when it beats the best
 * source-group one by 5%) and recomputes the forces with it.  result_host (nullable, 8 doubles) = {delta_scale,
 * warps_per_block, mid_slots, warps_per_sm, lpt_order, ms per force evaluation, warps_per_source, wide_registers};
 * the chosen lane width, split and pass group sizes are read with cssg_system_lanes, cssg_system_lane_split and
 * cssg_system_pass_groups.  Synchronises the context's stream. */
int cssg_system_autotune(cssg_system* sys, int reps, double* result_host);
/* The reference throws at the first failing walk or geodesic (ERRORERROR, inc/debuggingHelp.h:19-31); here failures
 * are collected. Error summary since the last call (synchronises): OR of (1 << CSSG_ST_*) over walks and sources,
 * and counters out_host[4] = {walk crossings, windows processed, vertex launches, in-range pairs} (nullable). */
int cssg_system_check(cssg_system* sys, int* status_bits, unsigned long long* counters_host);
/* simpleModel's neighbors / neighborDistances / neighborVectors (simpleModel.h:75-79, filled by findNeighbors,
 * simpleModel.cpp:68-112): pair data of the last force evaluation, host arrays with capacity cap: source i, target j,
 * distance, start tangent (3).  Returns the number of candidate pairs in *count (which may exceed cap).  The first
 * call switches pair recording on (later force evaluations record) and returns 0 pairs. */
int cssg_system_pairs(cssg_system* sys, int cap, int* i_host, int* j_host, double* d_host, double* t_host, int* count);
/* noseHooverNVT's bathVariables (noseHooverNVT.h:39-40) plus its KE and scale: Nose-Hoover chain state, per
 * system: (M+1) x 4 bath variables + {kinetic energy, scale factor}, host array of K * (4 (M+1) + 2) doubles. */
int cssg_system_chain(cssg_system* sys, double* chain_host, int capacity);
/* No reference counterpart (profiling). Timing of the last step() call: milliseconds of the dominant kernel
 * (geodesic+force) and of the walk, from CUDA events on the system stream (filled when timing is enabled with
 * cssg_system_timing(sys, 1)). */
int cssg_system_timing(cssg_system* sys, int enable);
int cssg_system_last_times(cssg_system* sys, double* ms_host, int capacity);
/* No reference counterpart. Learned screen for the system's force pass (cell-list systems): enable = 1 uploads
 * params_host (cssg_mlp_param_count() FP32 values) and skips candidate pairs whose predicted distance |chord| +
 * sigma * yhat exceeds sigma * (1 + margin); their faces still complete the reference patch, so the patch and every
 * computed distance stay exact. enable = 0 returns to the plain exact path. */
int cssg_system_set_screen(cssg_system* sys, const float* params_host, double margin, int enable);
/* No reference counterpart. Screen counters since the last call: out_host[3] = {candidate pairs, screened-out pairs,
 * tensor-core wait failures}. Synchronises and resets. */
int cssg_system_screen_counters(cssg_system* sys, unsigned long long* out_host);
/* No reference counterpart.  Regular propagation pass with one source per lane: lanes_per_warp = 16 or 32 sources
 * share a warp, each lane solving its own source (every FP64 instruction then serves up to 32 sources; the pass for
 * many small patches), 0 = source groups of cssg_system_set_tuning's warps_per_source.  Results are the same either
 * way; sources whose tables overflow are redone by the medium and large source-group passes.  Needs the cell-list
 * neighbour structure (range > 0).  With this pass, set_tuning's lpt_order = 1 sorts each run of 256 consecutive
 * sources of the cell order by their last cost, largest first (sources a warp takes together then cost about the
 * same and stay close on the mesh).  cssg_system_autotune also tries both lane widths and keeps the fastest choice;
 * cssg_system_lanes reports the current one.  Drops the captured step graph. */
int cssg_system_set_lanes(cssg_system* sys, int lanes_per_warp);
int cssg_system_lanes(cssg_system* sys, int* lanes_per_warp);
/* No reference counterpart.  With the lane pass on: the group_sources costliest sources of the last force evaluation
 * (ordered longest first by cost) are solved by the source-group pass first and the rest by the lane pass (a long
 * source fills a group's lanes; a warp of lanes waits for its longest source).  0 = the lane pass takes every
 * source.  Results are the same either way.  cssg_system_autotune tries 0 and 1/64, 1/16 and 1/4 of the sources.
 * Drops the captured step graph. */
int cssg_system_set_lane_split(cssg_system* sys, int group_sources);
/* No reference counterpart.  Warps per source of the medium and large propagation passes (the sources whose tables
 * or caps overflow the regular pass: the largest patches), 1, 2, 4 or 8; 0 = the regular pass's warps_per_source.
 * A few huge patches are often the tail of a force evaluation, and more warps per source shorten it.  The autotuner
 * tries (0, 0), (8, 0) and (8, 8) after choosing the rest.  Results do not depend on it.  Drops the step graph. */
int cssg_system_set_pass_groups(cssg_system* sys, int medium_warps, int large_warps);
int cssg_system_pass_groups(cssg_system* sys, int* medium_warps, int* large_warps);
int cssg_system_lane_split(cssg_system* sys, int* group_sources);
/* No reference counterpart (diagnostics).  Work of each source in the last force evaluation (windows processed +
 * vertex launches + 1, and 8 per round in the group pass): host array of at least the system's particle count. */
int cssg_system_source_costs(cssg_system* sys, int capacity, int* cost_host);
/* No reference counterpart (the reference's propagation and walk loops are unbounded, and a failing walk throws:
 * triangulatedMeshSpace.cpp:474, :534-541).  Per-source work caps of the three propagation passes, in windows
 * processed: a source that exceeds the regular pass's cap (or its tables) is redone by the medium pass, then by the
 * large pass; past the large pass's cap it reports CSSG_ST_CAPACITY (cssg_system_check).  Values <= 0 keep the
 * current cap (set at creation from the expected patch size).  Drops the captured step graph. */
int cssg_system_set_work_caps(cssg_system* sys, int regular, int medium, int large);
/* No reference counterpart. Periodic exact audit of the learned screen: with every > 0, every every-th step of
 * cssg_system_step runs the screened force pass and the plain exact pass on the same positions.  The exact pass
 * drives that step (its forces, kicks and pair records), so an audited step is always exact; a source whose screened
 * pass found fewer in-range pairs (d <= sigma) than the exact one means the screen dropped an in-range pair, and then
 * the screen switches itself off on the device: later force passes keep every candidate pair (the plain exact
 * results) until cssg_system_set_screen(..., enable = 1) is called again.  every = 0 turns the audit off.  Steps
 * between audits are not checked.  Drops the captured step graphs. */
int cssg_system_set_screen_audit(cssg_system* sys, int every);
/* No reference counterpart. out_host[3] = {audits run, sources that lost an in-range pair to the screen in an audit,
 * 1 if an audit has switched the screen off}, cumulative since the screen was enabled.  Synchronises. */
int cssg_system_screen_audit_status(cssg_system* sys, long long* out_host);
/* No reference counterpart.  Number of kernels one step() launches (the integrator's fixed sequence).  A step that
 * audits the screen launches the longest-first ordering kernels (0, 1 or 3) + 4 more. */
int cssg_system_kernels_per_step(cssg_system* sys, int* count);
/* No reference counterpart.  Kernels of a step that audits the screen (the same as cssg_system_kernels_per_step
 * when the audit is off). */
int cssg_system_kernels_per_audit_step(cssg_system* sys, int* count);

/* ---- diagnostics ------------------------------------------------------------------------------------------------
 * No reference counterpart.  Measured FP64 fused-multiply-add issue rate of the device (GFLOP/s, 2 flops per FMA),
 * from a register-resident dependent-chain kernel timed with CUDA events on the context stream; the denominator of
 * the FP64 roofline of the geodesic kernel.  Synchronises. */
int cssg_diag_fp64_peak(cssg_ctx* ctx, double* gflops_host);
/* FP64 flops of one processed window of the exact propagation on its usual path (trim, the opposite vertex's
 * proposal, two children), counted from the code once (window.cuh); the propagation's FP64 roofline is windows
 * processed x this figure. */
int cssg_diag_flops_per_window(void);
/* The reciprocal the propagation uses for geometric denominators (Newton-Raphson from a float seed), on n device
 * doubles: out[i] = 1/x[i] within a few ulps.  For accuracy tests. */
int cssg_diag_reciprocal(cssg_ctx* ctx, int n, const double* x, double* out);

/* ---- learned distance screen -------------------------------------------------------------------------------
 * No counterpart in the reference: a 14 -> 64 -> 64 -> 64 -> 1 GELU MLP that predicts the normalised geodesic
 * excess (d - |chord|) / sigma of a candidate pair, so that pairs predicted beyond sigma plus a calibrated margin can
 * skip exact propagation.  Parameters are one FP32 array of cssg_mlp_param_count() values:
 * W1[64][16] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] w4[64] b4 (W rows = output units). */
int cssg_mlp_param_count(void);
/* Features of pairs (pi[p] -> pj[p]) of particles on one mesh: X_bf16[nPairs][16] (14 features + 2 zeros, BF16)
 * and |chord| / sigma (nullable).  face[], pos[3*] are the particles' faces and R3 positions. */
int cssg_screen_features(cssg_ctx* ctx, const cssg_mesh* mesh, double sigma, int nPairs, const int* pi, const int* pj,
                         const int* face, const double* pos, void* X_bf16, float* chord_over_sigma);
/* Inference on the tensor cores (tcgen05, BF16 operands, FP32 accumulation in tensor memory): y[n].  X_bf16 must be
 * 16-byte aligned (rows are read as 16-byte words; else CSSG_ERR_ARG).  err_flag (nullable, device int) is set to 1
 * if a tensor-core completion wait timed out. */
int cssg_mlp_infer(cssg_ctx* ctx, const void* X_bf16, int n, const float* params, float* y, int* err_flag);
/* Gradient of 0.5 sum_p (f(x_p) - y_p)^2 with respect to params (FP32 forward/backward with the BF16 roundings of
 * inference): grad[cssg_mlp_param_count()] is overwritten; loss (nullable) receives the sum. */
int cssg_mlp_grad(cssg_ctx* ctx, const void* X_bf16, const float* y, int n, const float* params, float* grad,
                  float* loss);
/* One Adam step (lr, beta 0.9 / 0.999) on params using grad / batch; m, v: zero-initialised state arrays. */
int cssg_mlp_adam(cssg_ctx* ctx, float* params, const float* grad, float* m, float* v, int batch, float lr, int step);

#ifdef __cplusplus
}
#endif
#endif /* CSSG_H */
