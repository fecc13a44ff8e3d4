/* refexec_harness.cpp -- drives the reference's own kernel code on the CPU.  TEST
 * INFRASTRUCTURE ONLY (it pins the oracle to the reference's own kernels; never shipped).
 *
 * build_refexec.py compiles this file after the reference's kernel headers, in one translation
 * unit, with refexec_shim.h in front.  The harness restates only the host glue the reference
 * keeps in files that need OpenGL or its config singleton:
 *  - initializeFrame's parameter derivation and launch sizes (kernel/Initialize.h:34-85);
 *  - the shared-texture set-up of Particles.cc:33-53 and initializeShared (Initialize.h:92-116),
 *    here plain host arrays behind the shim's surfaces;
 *  - Communication::addParticlesCallback (Communication.h:637-655), writing the surfaces
 *    directly instead of through staging buffers and a kernel;
 *  - the call sequence of Fluid::compute (Fluid.cu:14-97).
 * Every kernel and every launcher it calls is the reference's own code.  Threads run in grid
 * order; solveCollisions runs with its atomic adds applied after the launch and
 * computeViscosity with its surface writes applied after the launch (every thread reads the
 * state from before the launch -- one legal schedule of those racy kernels).
 */
#include "pbd.h"

namespace refx {
uint3 g_threadIdx, g_blockIdx;
dim3 g_blockDim, g_gridDim;
bool defer_atomics = false, defer_surface_writes = false;
std::vector<FloatAdd> atomic_log;
std::vector<SurfWrite> surface_log;

struct Host {
    pbd_params prm;
    unsigned width = 0, capacity = 0, N = 0;
    std::vector<float4> tex[8];      // positions, predicted, velocities, colors, and their copies
    std::vector<float4> buf[10];     // d_positions ... d_colorsCopy (Particles.cc:44-53)
    bool live = false;
};
Host H;

void setup_frame() {   // Initialize.h:27-85 with the config values taken from pbd_params
    const pbd_params& p = H.prm;
    simulationParameters.numberOfParticles = H.N;
    simulationParameters.textureWidth = H.width;
    simulationParameters.maxNeighboursPerParticle = p.max_neighbours_per_particle;
    simulationParameters.maxContactConstraints = simulationParameters.maxNeighboursPerParticle * simulationParameters.numberOfParticles;
    simulationParameters.maxGrid = p.max_grid;
    simulationParameters.maxParticles = H.capacity;
    simulationParameters.maxPossibleContactConstraints = simulationParameters.maxNeighboursPerParticle * simulationParameters.maxParticles;
    simulationParameters.particleRadius = p.particle_radius;
    simulationParameters.particleDiameter = 2.0f * simulationParameters.particleRadius;
    simulationParameters.kernelWidthSpiky = simulationParameters.particleDiameter * p.kernel_width_spiky;
    simulationParameters.restDensity = p.rest_density;
    simulationParameters.kSCorr = p.k_scorr;
    simulationParameters.nSCorr = p.n_scorr;
    simulationParameters.qSCorr = simulationParameters.kernelWidthSpiky * p.q_scorr;
    simulationParameters.eVorticity = p.e_vorticity;
    simulationParameters.kernelWidthPoly = p.kernel_width_poly;
    simulationParameters.cViscosity = p.c_viscosity;
    simulationParameters.deltaT = p.delta_t;
    simulationParameters.gravity = p.gravity;
    simulationParameters.kernelWidthNeighbours = p.kernel_width_neighbours;
    simulationParameters.stiffness = p.stiffness;
    simulationParameters.enclosureVelocityDamping = p.enclosure_velocity_damping;
    simulationParameters.enclosurePositionDamping = p.enclosure_position_damping;
    simulationParameters.bounds.x.min = p.bounds_min[0];
    simulationParameters.bounds.x.max = p.bounds_max[0];
    simulationParameters.bounds.y.min = p.bounds_min[1];
    simulationParameters.bounds.y.max = p.bounds_max[1];
    simulationParameters.bounds.z.min = p.bounds_min[2];
    simulationParameters.bounds.z.max = p.bounds_max[2];
    params = simulationParameters;   // cudaMemcpyToSymbol(params, ...)
    const unsigned tpb = p.threads_per_block;
    cudaCallParameters.blocksForParticleBased = dim3((unsigned)std::ceil(simulationParameters.numberOfParticles / (float)tpb), 1, 1);
    cudaCallParameters.threadsForParticleBased = dim3(tpb, 1, 1);
    cudaCallParameters.blocksForContactBased = dim3((unsigned)std::ceil(simulationParameters.maxContactConstraints / (float)tpb), 1, 1);
    cudaCallParameters.threadsForContactBased = dim3(tpb, 1, 1);
    cudaCallParameters.blocksForGridBased = dim3((unsigned)std::ceil(simulationParameters.maxGrid / (float)tpb), 1, 1);
    cudaCallParameters.threadsForGridBased = dim3(tpb, 1, 1);
    cudaCallFullRangeParameters.blocksForAllParticlesPossibleBased = dim3((unsigned)std::ceil(simulationParameters.maxParticles / (float)tpb), 1, 1);
    cudaCallFullRangeParameters.threadsForAllParticlesPossibleBased = dim3(tpb, 1, 1);
}
}  // namespace refx

extern "C" {

int refx_create(const pbd_params* prm, unsigned width) {
    using namespace refx;
    if (H.live) return 1;
    H.prm = *prm;
    H.width = width;
    H.capacity = width * width;
    H.N = 0;
    for (auto& t : H.tex) t.assign(H.capacity, make_float4(0, 0, 0, 0));
    for (auto& b : H.buf) b.assign(H.capacity, make_float4(0, 0, 0, 0));
    surface<void, cudaSurfaceType2D>* s[8] = {&positions4, &predictedPositions4, &velocities4, &colors4,
                                              &positions4Copy, &predictedPositions4Copy, &velocities4Copy, &colors4Copy};
    for (int k = 0; k < 8; ++k) { s[k]->data = H.tex[k].data(); s[k]->width = width; }
    float4** b[10] = {nullptr, &deviceBuffers.d_positions, &deviceBuffers.d_predictedPositions, &deviceBuffers.d_velocities,
                      &deviceBuffers.d_colors, nullptr, &deviceBuffers.d_positionsCopy, &deviceBuffers.d_predictedPositionsCopy,
                      &deviceBuffers.d_velocitiesCopy, &deviceBuffers.d_colorsCopy};
    for (int k = 0; k < 10; ++k) if (b[k]) *b[k] = H.buf[k].data();
    setup_frame();
    initializeSortReorder();     // SortReorder.h:221-238 (resetCellInfo once, identity particle ids)
    initializeCollision();       // Collision.h:470-476
    initializeDensity();         // Density.h:321-330
    H.live = true;
    return 0;
}

void refx_destroy(void) {
    using namespace refx;
    if (!H.live) return;
    cleanupSortReorder();
    cleanupCollision();
    cleanupDensity();
    H.live = false;
}

int refx_add_particles(unsigned n, const float* pos4, const float* vel4, const float* col4) {
    using namespace refx;
    if (H.N + n > H.capacity) return 2;
    for (unsigned k = 0; k < n; ++k) {
        const unsigned i = H.N + k;
        H.tex[0][i] = make_float4(pos4[4 * k], pos4[4 * k + 1], pos4[4 * k + 2], pos4[4 * k + 3]);
        H.tex[2][i] = make_float4(vel4[4 * k], vel4[4 * k + 1], vel4[4 * k + 2], vel4[4 * k + 3]);
        if (col4) H.tex[3][i] = make_float4(col4[4 * k], col4[4 * k + 1], col4[4 * k + 2], col4[4 * k + 3]);
    }
    H.N += n;
    return 0;
}

/* phase 0: whole frame; 1: stop after computeCellInfo; 2: stop after findNeighbours */
int refx_step_phase(int phase) {
    using namespace refx;
    const pbd_params& p = H.prm;
    setup_frame();                                       // initializeFrame
    if (H.N == 0) return 0;                              // Fluid.cu:19
    if (p.collision_type > 1) return 6;
    const bool batches = p.collision_type == 1;
    if (p.active & PBD_ACTIVE_APPLY_FORCES) cudaCallApplyForces();
    cudaCallInitializeCellIds();
    sortIds();
    reorderStorage();
    cudaCallResetCellInfo();
    cudaCallComputeCellInfo();
    if (phase == 1) return 0;
    if (batches) cudaCallResetContacts();                // Fluid.cu:37-39
    if (p.active & PBD_ACTIVE_FIND_CONTACTS) cudaCallFindContacts();
    if (p.active & PBD_ACTIVE_FIND_NEIGHBOURS) cudaCallFindNeighbours();
    if (phase == 2) return 0;
    for (unsigned it = 0; it < p.solver_iterations; ++it) {
        if (p.active & PBD_ACTIVE_COMPUTE_LAMBDA) cudaCallComputeLambda();
        if (p.active & PBD_ACTIVE_COMPUTE_DELTA_POSITIONS) cudaCallComputeDeltaPositions();
        for (unsigned k = 0; k < p.stabilization_iterations; ++k) {
            if (!batches) {
                defer_atomics = true;
                cudaCallSolveCollisions();
                defer_atomics = false;
                continue;
            }
            // Fluid.cu:62-72.  Threads run one after another in grid order, so each batch is the
            // greedy matching of the pending list entries in index order -- one legal schedule of
            // setupCollisionConstraintBatches (whose blocks race and whose __syncthreads sits in
            // divergent code, Collision.h:359-369); it agrees with every other schedule on scenes
            // where each particle has at most one partner.
            cudaCallResetContactConstraintSuccess();
            for (unsigned b = 0; b < p.max_collision_batches; ++b) {
                cudaCallResetContactConstraintParticleUsed();
                cudaCallSetupCollisionConstraintBatches();
                cudaCallSetupCollisionConstraintBatchesCheck();
            }
        }
        if (p.active & PBD_ACTIVE_APPLY_DELTA_POSITIONS) cudaCallApplyDeltaPositions();
    }
    if (p.active & PBD_ACTIVE_UPDATE_POSITIONS) cudaCallUpdatePositions();
    if (p.active & PBD_ACTIVE_COMPUTE_OMEGAS) cudaCallComputeOmegas();
    if (p.active & PBD_ACTIVE_COMPUTE_VORTICITY) cudaCallComputeVorticity();
    if (p.active & PBD_ACTIVE_COMPUTE_VISCOSITY) {
        defer_surface_writes = true;
        cudaComputeViscosity();
        defer_surface_writes = false;
    }
    return 0;
}

unsigned refx_num_particles(void) { return refx::H.N; }

static void out4(const float4* a, float* o, unsigned n) {
    for (unsigned i = 0; i < n; ++i) { o[4 * i] = a[i].x; o[4 * i + 1] = a[i].y; o[4 * i + 2] = a[i].z; o[4 * i + 3] = a[i].w; }
}

void refx_get_state(float* x4, float* v4, float* p4, float* col4) {
    using namespace refx;
    if (x4) out4(H.tex[0].data(), x4, H.N);
    if (p4) out4(H.tex[1].data(), p4, H.N);
    if (v4) out4(H.tex[2].data(), v4, H.N);
    if (col4) out4(H.tex[3].data(), col4, H.N);
}

void refx_get_debug(unsigned* keys, unsigned* perm, unsigned* cell_start, unsigned* cell_end, unsigned ncells,
                    float* lambda, float* fext4, float* omega4) {
    using namespace refx;
    const unsigned N = H.N;
    if (keys) memcpy(keys, d_cellIds_out, N * 4u);
    if (perm) memcpy(perm, d_particleIds_out, N * 4u);
    if (ncells > H.prm.max_grid) ncells = H.prm.max_grid;
    if (cell_start) memcpy(cell_start, d_cellStarts, (size_t)ncells * 4);
    if (cell_end) memcpy(cell_end, d_cellEndings, (size_t)ncells * 4);
    if (lambda) memcpy(lambda, d_lambdas, N * 4u);
    if (fext4) out4(d_externalForces, fext4, N);
    if (omega4) for (unsigned i = 0; i < N; ++i) {
        omega4[4 * i] = d_omegas[i].x; omega4[4 * i + 1] = d_omegas[i].y; omega4[4 * i + 2] = d_omegas[i].z; omega4[4 * i + 3] = 0.f;
    }
}

void refx_get_neighbours(unsigned max_entries, unsigned* list, unsigned* count, unsigned* contacts) {
    using namespace refx;
    const unsigned N = H.N, M = H.prm.max_neighbours_per_particle;
    for (unsigned i = 0; i < N; ++i) {
        const unsigned c = d_neighbourCounters[i];
        if (count) count[i] = c;
        if (contacts) contacts[i] = d_contactCounters[i];
        if (list) {
            const unsigned m = c < max_entries ? c : max_entries;
            memcpy(list + (size_t)i * max_entries, d_neighbours + (size_t)i * M, m * 4u);
        }
    }
}

}  // extern "C"
