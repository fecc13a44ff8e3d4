/*
 * pbd.h -- C ABI of the GB300-native unified-particle PBD step.
 *
 * This library replaces the per-frame step of niklasandersson/PBD-Simulation-Framework-CUDA:
 * `Fluid::compute()` (src/app/simulation/Fluid.cu:14-97) and the kernels it drives
 * (src/app/simulation/kernel/{Forces,Hash,SortReorder,Collision,Density,Update}.h).
 * The reference exposes that step as a C++ class behind `Cuda_Computable::compute()`
 * (src/cuda/Cuda_Computable.h:8-23) plus parameterless launchers (kernel/Kernels.h:18-43)
 * that read a global `__constant__ SimulationParameters params` (kernel/Globals.h:50-77)
 * filled from config.txt every frame (kernel/Initialize.h:20-86).  Here the same step is
 * one handle-based C API: plain pointers and sizes, no CUDA or torch types in the
 * signatures (streams are passed as `void*` holding a cudaStream_t).
 *
 * Conventions
 *  - Every function returns an int status (PBD_OK == 0) and never throws; the text of the
 *    last error on the calling thread is returned by pbd_last_error().
 *  - Particle state is float4 per particle (x, y, z, w), stored as 4 consecutive floats.
 *  - A pbd_sim handle is externally synchronised: one host thread at a time.  Separate
 *    handles are independent.  All GPU work of a call is queued on the stream passed to
 *    it (NULL = the legacy default stream) and is asynchronous unless stated otherwise.
 *    A handle remembers the stream of its last call and, when the next call comes on
 *    another stream, first waits for that one: keep a stream alive until the handle's
 *    next call (or pbd_sync) after the last use of it.
 *  - Particles are kept in Morton-sorted order, exactly as the reference re-orders its
 *    textures every frame (kernel/SortReorder.h:86-129); pbd_get_state returns that order.
 */
#ifndef PBD_H
#define PBD_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBD_ABI_VERSION 1u

/* ---- status codes ---------------------------------------------------------------- */
#define PBD_OK                0
#define PBD_ERR_INVALID_ARG   1  /* null pointer, bad size, bad enum */
#define PBD_ERR_CAPACITY      2  /* N + n would exceed the capacity given to pbd_create */
#define PBD_ERR_CUDA          3  /* a CUDA runtime call failed (text in pbd_last_error) */
#define PBD_ERR_CONFIG        4  /* config.txt could not be read or parsed */
#define PBD_ERR_TIMEOUT       5  /* a bounded device-side wait gave up (no hang, no trap) */
#define PBD_ERR_UNSUPPORTED   6  /* a valid reference option this library does not implement */
#define PBD_ERR_ALLOC         7  /* device or host allocation failed */
#define PBD_ERR_RANGE         8  /* a parameter is outside the range the reference's setters accept */

/* ---- Active flags: Application.Simulation.Active.* (config.txt:40-52, Fluid.cu:21-96) ---- */
#define PBD_ACTIVE_APPLY_FORCES            (1u << 0)
#define PBD_ACTIVE_FIND_CONTACTS           (1u << 1)
#define PBD_ACTIVE_FIND_NEIGHBOURS         (1u << 2)
#define PBD_ACTIVE_COMPUTE_LAMBDA          (1u << 3)
#define PBD_ACTIVE_COMPUTE_DELTA_POSITIONS (1u << 4)
#define PBD_ACTIVE_APPLY_DELTA_POSITIONS   (1u << 5)
#define PBD_ACTIVE_UPDATE_POSITIONS        (1u << 6)
#define PBD_ACTIVE_COMPUTE_OMEGAS          (1u << 7)
#define PBD_ACTIVE_COMPUTE_VORTICITY       (1u << 8)
#define PBD_ACTIVE_COMPUTE_VISCOSITY       (1u << 9)
#define PBD_ACTIVE_ALL                     0x3FFu

/* ---- behaviour flags (pbd_params.flags) ------------------------------------------- */
/* Reproduce kernel/SortReorder.h:183-184: at i == N-1 the reference writes
 * cellEndings[N-1] = N (indexing by particle, not by cell).  When cell number N-1 is
 * occupied and is not the last cell, its range then runs to N.  On by default. */
#define PBD_FLAG_CELL_END_QUIRK  (1u << 0)
/* Carry a uint32 particle id through every re-order so callers can follow particles. */
#define PBD_FLAG_TRACK_IDS       (1u << 1)
/* Carry the per-particle colour array through every re-order (kernel/SortReorder.h:106-107)
 * and write colour = neighbourCount / maxNeighbours as findNeighbours does
 * (kernel/Collision.h:118-120).  Off by default: colours are cosmetic. */
#define PBD_FLAG_COLORS          (1u << 2)
/* Walk the cells in every neighbour pass.  By default a pass that walks the cells (lambda,
 * omega) keeps, per particle and in list order, the entries within the kernel cut at the
 * positions it read, and the pass after it at the same positions (delta, viscosity without
 * vorticity) reads only those; the entries left out add exact zeros there, so both ways give
 * identical results: this flag exists for testing and measurement. */
#define PBD_FLAG_FULL_WALK       (1u << 3)
/* The later lambda passes and the delta passes copy each block's neighbourhood (the particles of
 * every cell its members' lists reach) into shared memory and walk it there instead of reading
 * the stored lists; the results are the same bits.  Measured slower than the stored lists on
 * GB300 (kept for testing and measurement).  Bit 4 is reserved. */
#define PBD_FLAG_STAGED_PASSES   (1u << 5)

/* ---- parameters: mirrors SimulationParameters (kernel/Globals.h:50-75) plus the
 *      config keys Fluid::compute reads directly (Fluid.cu:35-67).  Field comments give
 *      the config.txt key under Application.Simulation unless stated otherwise. -------- */
typedef struct pbd_params {
    uint32_t struct_size;                 /* = sizeof(pbd_params); set by pbd_params_default */
    uint32_t threads_per_block;           /* Application.Cuda.threadsPerBlock (advisory)      */
    float    particle_radius;             /* Particles.particleRadius; diameter = 2 r          */
    uint32_t max_neighbours_per_particle; /* Particles.maxNeighboursPerParticle (list cap M)   */
    float    delta_t;                     /* Forces.deltaT                                      */
    float    gravity;                     /* Forces.gravity (y component)                       */
    float    rest_density;                /* Density.restDensity                                */
    float    kernel_width_spiky;          /* Density.kernelWidthSpiky, x particle diameter      */
    float    k_scorr;                     /* Density.kSCorr                                     */
    int32_t  n_scorr;                     /* Density.nSCorr                                     */
    float    q_scorr;                     /* Density.qSCorr, x spiky width                      */
    float    c_viscosity;                 /* Viscosity.cViscosity                               */
    float    kernel_width_poly;           /* Viscosity.kernelWidthPoly (absolute)               */
    float    e_vorticity;                 /* Vorticity.eVorticity                               */
    uint32_t collision_type;              /* Collision.collisionType (0 = per-contact Jacobi)   */
    uint32_t kernel_width_neighbours;     /* Collision.kernelWidthNeighbours (cell shells)      */
    uint32_t max_collision_batches;       /* Collision.maxCollisionBatches                      */
    float    stiffness;                   /* Collision.stiffness                                */
    float    enclosure_position_damping;  /* Enclosure.enclosurePositionDamping                 */
    float    enclosure_velocity_damping;  /* Enclosure.enclosureVelocityDamping                 */
    float    bounds_min[3];               /* Enclosure.{X,Y,Z}.min                              */
    float    bounds_max[3];               /* Enclosure.{X,Y,Z}.max                              */
    uint32_t solver_iterations;           /* Iterations.solverIterations                        */
    uint32_t stabilization_iterations;    /* Iterations.stabilizationIterations                 */
    uint32_t active;                      /* PBD_ACTIVE_* bitmask (Active.*)                    */
    uint32_t max_grid;                    /* Morton cells addressable; 128^3 (Particles.cc:8)   */
    float    lambda_epsilon;              /* relaxation eps of lambda = -C/(B+C+eps); 1e-4 (Density.h:90) */
    uint32_t flags;                       /* PBD_FLAG_* bitmask                                 */
} pbd_params;

typedef struct pbd_sim pbd_sim;

/* ---- parameters ------------------------------------------------------------------ */
/* Fill *p with the values of the reference's config.txt (config.txt:9-131). */
int pbd_params_default(pbd_params* p);
/* Parse a config file in the reference's grammar (src/parser/ConfigParser.h:265-330 with
 * comments, #define and #include) and overwrite the fields whose keys it holds.  Replaces
 * Config::getInstance(file) + the getValue calls of kernel/Initialize.h:33-73. */
int pbd_load_config(pbd_params* p, const char* path);
/* Same, from an in-memory text.  `base_dir` resolves #include (may be NULL). */
int pbd_parse_config(pbd_params* p, const char* text, const char* base_dir);
/* Write *p as a config file in the reference's layout (ConfigParser.h:241-247). */
int pbd_write_config(const pbd_params* p, const char* path);
/* Check every field against the ranges of the reference's setters
 * (kernel/Communication.h:440-624); PBD_ERR_RANGE names the first bad field. */
int pbd_validate_params(const pbd_params* p);

/* ---- lifecycle ------------------------------------------------------------------- */
/* Replaces Fluid::Fluid() -> cudaInitializeKernels() (kernel/Initialize.h:122-130).
 * `capacity` plays the role of maxParticles = textureWidth^2 (Particles.cc:12).
 * Allocates every device buffer once; the step itself never allocates. */
int pbd_create(const pbd_params* p, uint32_t capacity, pbd_sim** out);
/* Replaces Fluid::~Fluid() -> cudaCleanupKernels() (kernel/Initialize.h:136-140). */
int pbd_destroy(pbd_sim* sim);
int pbd_set_params(pbd_sim* sim, const pbd_params* p);   /* validated like pbd_validate_params */
int pbd_get_params(const pbd_sim* sim, pbd_params* p);
int pbd_num_particles(const pbd_sim* sim, uint32_t* n);
int pbd_capacity(const pbd_sim* sim, uint32_t* cap);

/* ---- particle injection (kernel/Communication.h:22-67, 626-660) ------------------- */
/* addParticlesCallback: append n particles at index N from host arrays of n float4
 * (col may be NULL).  Rejected with PBD_ERR_CAPACITY when N + n > capacity (the reference
 * returns silently).  Synchronous with respect to the host arrays, except when they are the
 * arrays pbd_step_readback returned (with col NULL): that copy is queued, and the library's
 * next write into those arrays comes after it. */
int pbd_add_particles(pbd_sim* sim, uint32_t n, const float* pos4, const float* vel4,
                      const float* col4);
/* Same, with a per-particle inverse mass (unified solids).  The reference forces mass 1
 * everywhere (Forces.h:75,94; Collision.h:223-224) while its collision code weighs the overlap
 * by inverseMass1 / (inverseMass1 + inverseMass2) (Collision.h:225): here that weight uses the
 * given inverse masses, a particle with inverse mass 0 (a solid) takes no gravity, external
 * force, density correction or viscosity, and all particles added without this call have
 * inverse mass 1 -- the reference's behaviour. */
int pbd_add_particles_mass(pbd_sim* sim, uint32_t n, const float* pos4, const float* vel4,
                           const float* col4, const float* inv_mass);
/* Same as pbd_add_particles, from device pointers (no host copy); queued on `stream`. */
int pbd_add_particles_device(pbd_sim* sim, uint32_t n, const float* d_pos4,
                             const float* d_vel4, const float* d_col4, void* stream);
/* addParticleCallback: one particle at pos with velocity 50*dir, w = 0. */
int pbd_add_particle(pbd_sim* sim, const float pos[3], const float dir[3]);
/* clearParticlesCallback: N = 0. */
int pbd_clear(pbd_sim* sim);

/* ---- the step -------------------------------------------------------------------- */
/* Run `nsteps` frames of Fluid::compute() (Fluid.cu:14-97) on `stream` (a cudaStream_t,
 * NULL = legacy default stream).  The whole frame is one CUDA graph launch; nothing is
 * synchronised, except that when the sim's previous call queued work on another stream the host
 * first waits for that stream.  Simulation::step's cudaDeviceSynchronize (Simulation.cu:16-19)
 * is pbd_sync(). */
int pbd_step(pbd_sim* sim, int nsteps, void* stream);
/* Wait for the sim's queued work and report device-side error words
 * (PBD_ERR_TIMEOUT if a bounded wait gave up). */
int pbd_sync(pbd_sim* sim);

/* ---- state out (synchronous; host pointers, any may be NULL) ------------------------ */
int pbd_get_state(pbd_sim* sim, float* pos4, float* vel4, float* pred4, uint32_t* ids);
/* No counterpart in the reference (its state never leaves the GPU).  pbd_step followed by the
 * positions and velocities of the final state, in host memory the library owns (pinned; valid
 * until the next pbd_step_readback, pbd_destroy or a pbd_add_particles from these same arrays
 * is complete): the position copy runs beside the last frame's omega / vorticity / viscosity
 * passes, and the viscosity pass stores the final velocities into that memory itself.
 * Synchronous.  nsteps >= 1; with no particles the arrays are returned unchanged. */
int pbd_step_readback(pbd_sim* sim, int nsteps, void* stream, const float** pos4, const float** vel4);
/* Device pointers of the current state buffers (valid until the next pbd_step/add/clear). */
int pbd_get_device_state(pbd_sim* sim, const float** d_pos4, const float** d_vel4,
                         const float** d_pred4);

/* ---- introspection for tests and tools -------------------------------------------- */
/* After a step: the sorted Morton keys, the sort permutation (index before the sort of
 * the particle now at i), cellStart/cellEnd for the first `ncells` cells, per-particle
 * lambda and f_ext (float4).  Any pointer may be NULL. */
int pbd_debug_dump(pbd_sim* sim, uint32_t* keys, uint32_t* perm, uint32_t* cell_start,
                   uint32_t* cell_end, uint32_t ncells, float* lambda, float* fext4,
                   float* omega4);
/* Materialise the neighbour list the reference would build this frame (findContacts +
 * findNeighbours, kernel/Collision.h:11-160): `list` is N x max_entries uint32, `count`
 * and `contacts` are N uint32.  Entries beyond max_entries are counted but not stored.
 * `walker` selects the traversal: 0 one thread per particle, 1 one warp per particle (the
 * path taken by particles whose list meets a very long cell range). */
int pbd_debug_neighbours(pbd_sim* sim, uint32_t max_entries, uint32_t* list,
                         uint32_t* count, uint32_t* contacts, int walker);
/* Run only the front of a frame: applyForces, initializeCellIds, sortIds, reorder,
 * resetCellInfo/computeCellInfo (Fluid.cu:21-33).  For bit-exact tests of keys,
 * permutation and cell ranges. */
int pbd_debug_front(pbd_sim* sim, void* stream);
/* Number of kernels one pbd_step frame launches (for launch accounting). */
int pbd_launches_per_step(pbd_sim* sim, uint32_t* n);
/* Run `nsteps` frames with direct launches (no graph) and a CUDA event pair around every
 * kernel; per kernel name, the launches and their summed device time.  For profiling only
 * (the reference has no counterpart: its only timer is an FPS counter,
 * src/glfw/GLFW_Window.cc:63-86). */
typedef struct pbd_kernel_stat {
    char     name[32];
    uint32_t launches;
    float    total_ms;
} pbd_kernel_stat;
int pbd_profile_frames(pbd_sim* sim, int nsteps, void* stream, pbd_kernel_stat* stats,
                       uint32_t max_stats, uint32_t* n_stats);

/* ---- tuning --------------------------------------------------------------------------- */
/* No counterpart in the reference (threads per block is a config value there,
 * Initialize.h:73).  Times the frame with 64, 128 and 256 threads per block for the neighbour
 * passes (3 frames each after 2 warm-up frames -- this ADVANCES the simulation by 15 frames) and
 * keeps the fastest.  With `cache_path` (a JSON-lines file) a result recorded for the same
 * workload signature is reused without measuring, and new results are appended. */
int pbd_autotune(pbd_sim* sim, const char* cache_path, void* stream, uint32_t* block);

/* ---- batched scenes ------------------------------------------------------------------ */
/* No counterpart in the reference (one scene per process there).  Many independent scenes
 * advance together: every kernel of a frame covers all scenes, so a frame is one graph launch
 * whatever the number of scenes.  Scenes share every parameter except the ones in
 * pbd_scene_desc.  Each scene's particles are sorted by (scene, Morton key) and use their own
 * 128^3-cell slice of the cell tables, so a scene evolves exactly as it would alone. */
typedef struct pbd_scene_desc {
    uint32_t capacity;          /* particles this scene may hold */
    float    rest_density;      /* Density.restDensity of this scene */
    float    gravity;           /* Forces.gravity of this scene */
    float    bounds_min[3];     /* Enclosure.{X,Y,Z}.min of this scene */
    float    bounds_max[3];     /* Enclosure.{X,Y,Z}.max of this scene */
} pbd_scene_desc;
typedef struct pbd_batch pbd_batch;
int pbd_batch_create(const pbd_params* shared, uint32_t nscenes, const pbd_scene_desc* scenes,
                     pbd_batch** out);
int pbd_batch_destroy(pbd_batch* batch);
int pbd_batch_add_particles(pbd_batch* batch, uint32_t scene, uint32_t n, const float* pos4,
                            const float* vel4);
int pbd_batch_step(pbd_batch* batch, int nsteps, void* stream);
int pbd_batch_sync(pbd_batch* batch);
int pbd_batch_num_particles(pbd_batch* batch, uint32_t scene, uint32_t* n);
/* The scene's particles in their current (Morton-sorted) order; arrays of
 * pbd_batch_num_particles float4.  Synchronous. */
int pbd_batch_get_state(pbd_batch* batch, uint32_t scene, float* pos4, float* vel4);
int pbd_batch_autotune(pbd_batch* batch, const char* cache_path, void* stream, uint32_t* block);
int pbd_batch_launches_per_step(pbd_batch* batch, uint32_t* n);
int pbd_batch_profile_frames(pbd_batch* batch, int nsteps, void* stream, pbd_kernel_stat* stats,
                             uint32_t max_stats, uint32_t* n_stats);

/* The density constraint after the last frame (no counterpart in the reference, whose density
 * lives inside computeLambda, Density.h:48-93): C_i = rho_i / rest_density - 1, rho_i the poly6
 * sum over particle i's list of the last frame (no self term) at the current positions.  `err`
 * (host, N floats, nullable) receives C_i in the current particle order; mean_abs and max_abs
 * the mean and maximum of |C_i| (nullable).  Needs a frame since the last add/clear
 * (PBD_ERR_INVALID_ARG otherwise); synchronises. */
int pbd_density_error(pbd_sim* sim, float* err, double* mean_abs, double* max_abs, void* stream);
/* The same C_i, averaged over the interior particles only: those whose list (the last frame's)
 * holds at least `min_neighbours` entries and whose current position lies more than `margin`
 * inside the enclosure on every axis -- the particles whose kernel support is filled with fluid
 * rather than cut by the free surface or a wall.  `counted` receives how many there were.
 * No counterpart in the reference; synchronises. */
int pbd_density_error_interior(pbd_sim* sim, uint32_t min_neighbours, float margin, double* mean_abs,
                               double* max_abs, uint32_t* counted, void* stream);

/* ---- headless particle sprites -------------------------------------------------------- */
/* The reference draws each particle as a shaded sphere sprite through OpenGL
 * (src/app/rendering/shader/particles/particleSpriteGeom.{vert,geom,frag}, Particles.cc:234-284).
 * This renders the same sprites without a graphics API, into an image:
 *  - colour per particle: mix((0.95, 0.97, 0.97), (0, 0, 1), colour.x^(1/6)) (.vert);
 *  - a quad of half-size sphere_radius around view * position, facing the camera (.geom);
 *  - per pixel inside the unit disc of the quad: normal (u, v, sqrt(1 - u^2 - v^2)) rotated back
 *    by the inverse of the view's rotation, Phong shading 0.3 ambient + 0.7 diffuse + 0.2 specular
 *    (exponent 10) with L = normalize(light_position - position), V = normalize(-view_direction),
 *    and the depth of the sphere surface 0.5 (z / w) + 0.5 (.frag); nearest fragment wins.
 * A pixel is covered when its centre lies in the quad's window rectangle [x0, x1) x [y0, y1);
 * colours are rounded to 8 bits.  Rows are returned top-down (row 0 = the window's top).
 * The matrices are column-major as glm and glUniformMatrix4fv(..., GL_FALSE, ...) use them; the
 * view's upper 3x3 must be a rotation (glm::lookAt).  The particle colours are the simulation's
 * colour array (PBD_FLAG_COLORS: neighbour count / maxNeighboursPerParticle). */
typedef struct pbd_camera {
    float view[16];            /* glm::lookAt (GLFW_Controls.cc:244) */
    float projection[16];      /* glm::perspective (GLFW_Controls.cc:69) */
    float view_direction[3];   /* world space (GL_Renderable.cc:34) */
    float light_position[3];   /* (0, 0, 10) in particleSpriteGeom.geom */
    float sphere_radius;       /* 0.5 in particleSpriteGeom.geom/.frag */
    uint32_t width, height;    /* pixels */
    float clear_rgba[4];       /* (0, 0, 0, 1) in GLFW_Window.cc:96 */
} pbd_camera;
/* rgba: width*height*4 bytes, depth: width*height floats (1 where no sprite); host pointers,
 * either may be NULL.  Allocates its image workspace on first use or when the size grows;
 * synchronises. */
int pbd_render_sprites(pbd_sim* sim, const pbd_camera* camera, uint8_t* rgba, float* depth, void* stream);

/* ---- adjoint ------------------------------------------------------------------------ */
/* No counterpart in the reference.  Gradients of a loss on the final positions of a rollout
 * with respect to the initial velocities and positions, the rest density and the relaxation
 * eps of lambda (pbd_params.lambda_epsilon).
 * pbd_adjoint_forward advances `nsteps` frames exactly as pbd_step does and keeps the state
 * every `ckpt_every` frames (device memory allocated here, not in the frame).
 * pbd_adjoint_backward takes dL/dx_final (host, N float4, in the order pbd_get_state returns
 * after the forward) and returns dL/dv0 and dL/dx0 (host, N float4, in the order of the state
 * before the forward; either may be NULL), dL/drest_density and dL/deps.  It recomputes each
 * segment from its checkpoint (the last one is taped by the forward itself) with the neighbour
 * lists, permutations and wall contacts of the forward held fixed (they are piecewise constant),
 * and leaves the simulation as the forward left it; it may be called again for another loss on
 * the same forward.  Supported: the density solve, contacts, walls, integration, omega +
 * vorticity confinement (its force reaches the next frame), XSPH viscosity and unified solids
 * (pbd_add_particles_mass), stabilizationIterations 0..8, enclosurePositionDamping; batches,
 * collisionType 1 and vorticity without computeOmegas return PBD_ERR_UNSUPPORTED. */
int pbd_adjoint_forward(pbd_sim* sim, int nsteps, int ckpt_every, void* stream);
int pbd_adjoint_backward(pbd_sim* sim, const float* dL_dx_final, float* dL_dv0, float* dL_dx0,
                         double* dL_drest_density, double* dL_deps, void* stream);

/* ---- sorting without allocation -------------------------------------------------- */
/* No counterpart in the reference.  For hosts that cannot call cudaMalloc where they sort
 * (engines that own all device memory from start-up, frame loops that must not stall on an
 * allocation): the step's stable radix sort of uint32 keys, with every byte of working memory
 * taken from one fixed array inside the library.  Inputs and outputs are the caller's device
 * buffers: d_keys_out receives the keys in ascending order of their low `key_bits` bits (1..32;
 * higher bits do not take part in the order, as with cub's end_bit) and d_perm_out the input
 * index of each output key (a stable sort, so keys equal in those bits keep their input order).
 * d_keys_out and d_perm_out must not overlap d_keys_in.
 * Limit: n <= 1,048,576 keys (the fixed array is 9,441,536 bytes and stays on every GPU that
 * loads the library until the process exits); larger n returns PBD_ERR_CAPACITY.  The first call
 * on each device looks up the array's device address (make it before any stream capture).  All
 * calls share the array: calls whose GPU work overlaps race and must be serialised by the
 * caller.  Asynchronous on `stream`; pbd_sort_noalloc_status reports how the last call ended. */
int pbd_sort_keys_noalloc(const uint32_t* d_keys_in, uint32_t* d_keys_out, uint32_t* d_perm_out,
                          uint32_t n, uint32_t key_bits, void* stream);
/* Waits for `stream` and returns PBD_ERR_TIMEOUT if the last pbd_sort_keys_noalloc on the current
 * device had a bounded look-back wait give up (its output is then not sorted), else PBD_OK. */
int pbd_sort_noalloc_status(void* stream);

/* ---- failure injection for tests (no counterpart in the reference) --------------------- */
/* After `skip` more device or pinned-host allocations of the library succeed, the next `fail`
 * allocations fail as on a GPU that is out of memory: the call that meets one returns
 * PBD_ERR_ALLOC and frees whatever it had taken.  (0, 0) switches it off.  Process-wide. */
int pbd_debug_fail_allocations(uint32_t skip, uint32_t fail);
/* The radix sort's look-back waits give up after `spins` polls (0 = the default, a few seconds)
 * and then set the device error word that pbd_sync (or pbd_sort_noalloc_status) reports as
 * PBD_ERR_TIMEOUT.  With hold_first_tile the first tile of every sort pass never publishes its
 * counts, so every wait on it runs out -- the failure path, exercised without a hang or a trap.
 * `sim` NULL sets the no-allocation sort's settings; otherwise the simulation's frames use them
 * from the next pbd_step or pbd_debug_front on. */
int pbd_debug_set_wait_limit(pbd_sim* sim, uint32_t spins, int hold_first_tile);

/* Text of the last error on this thread ("" if none). */
const char* pbd_last_error(void);
uint32_t pbd_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PBD_H */
