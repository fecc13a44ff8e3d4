// pbd_sim.cu -- the simulation handle, the frame schedule, CUDA-graph replay and the C ABI.
//
// Host-side counterpart of the reference's Fluid (src/app/simulation/Fluid.{h,cu}) and of
// the kernel module's host globals (kernel/Globals.h:15-37, kernel/Initialize.h):
//  - every device buffer is allocated once in pbd_create (one arena) -- the frame never
//    allocates, unlike the per-frame parameter upload of Initialize.h:71;
//  - a frame is recorded once into a CUDA graph and replayed per pbd_step call; the graph is
//    re-recorded only when N or the parameters change;
//  - multi-buffered arrays are addressed through a small "which buffer is current" record
//    (Cur).  Predicted positions have three buffers: the frame's anchor (p* right after the
//    re-order, which the neighbour cells are taken from for the whole frame, as the reference
//    builds its list once per frame) and two the solver passes alternate between.  A frame
//    moves the record through a short cycle; one graph is recorded per starting record and
//    the graphs are replayed in turn.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pbd_internal.h"
#include "pbd_kernels.cuh"
#include "pbd_staged.cuh"
#include "pbd_adjoint.cuh"
#include "pbd_contacts.cuh"
#include "pbd_sprites.cuh"

namespace pbd {
thread_local std::string g_last_error;
void set_error(const std::string& m) { g_last_error = m; }
void clear_error() { g_last_error.clear(); }

// Allocation-failure injection (pbd_debug_fail_allocations): `skip` more allocations succeed,
// then `fail` allocations fail.
static std::mutex g_alloc_mutex;
static uint32_t g_alloc_skip = 0, g_alloc_fail = 0;
static bool injected_failure() {
    std::lock_guard<std::mutex> lock(g_alloc_mutex);
    if (g_alloc_skip > 0) { --g_alloc_skip; return false; }
    if (g_alloc_fail > 0) { --g_alloc_fail; return true; }
    return false;
}
cudaError_t lib_malloc(void** p, size_t bytes) {
    if (injected_failure()) { *p = nullptr; return cudaErrorMemoryAllocation; }
    return cudaMalloc(p, bytes);
}
cudaError_t lib_host_alloc(void** p, size_t bytes, unsigned int flags) {
    if (injected_failure()) { *p = nullptr; return cudaErrorMemoryAllocation; }
    return cudaHostAlloc(p, bytes, flags);
}
}  // namespace pbd

using namespace pbd;

namespace {

struct Cur {
    int x = 0, p = 0, v = 0;   // current buffer of positions (also colours, ids), predictions, velocities
    bool operator==(const Cur& o) const { return x == o.x && p == o.p && v == o.v; }
};
constexpr int kMaxGraphs = 8;
// Stored list capacities (slot-major, only the used slots are touched).  A particle whose list
// is longer goes to the warp-cooperative cell walk.
constexpr uint32_t kListMax = 64;    // near list: entries within the cut
constexpr uint32_t kFullMax = 255;   // full list: every entry of the frame's list (meta holds 8-bit counts)
constexpr uint32_t kFullSlim = 128;  // the full list's slots when the list covers 27 cells (~32 entries)

constexpr int kThreadsParticle = 256;
constexpr int kThreadsNeighbourDefault = 128;
constexpr int kThreadsCoop = 128;         // 4 warps, one deferred particle per warp
constexpr uint32_t kCoopBlocks = 16;      // leading blocks of a list pass that walk its particles without a list

inline uint32_t div_up(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace

// What the adjoint keeps of one frame (device buffers of N entries each).
constexpr int kMaxTapeIters = 16;
constexpr int kMaxTapeStab = 8;   // stabilizationIterations the adjoint takes
struct Tape {
    float4* x_in;                  // state before applyForces (pre-sort order)
    float4* v_in;
    uint32_t* perm;                // sort permutation of the frame
    uint32_t* keys;                // sorted keys (rebuild the frame's cell tables)
    float4* p_it[kMaxTapeIters];   // p* entering each solver iteration (sorted order)
    float4* p_s[kMaxTapeIters][kMaxTapeStab];   // p* entering the iteration's contact passes 1..S-1
    float* lam[kMaxTapeIters];     // lambda of each iteration
    float4* aux[kMaxTapeIters];    // the lambda pass's sums (2N float4: rho, B, S)
    uint32_t* near[kMaxTapeIters];       // each iteration's near lists (kListMax x N, slot-major)
    uint32_t* near_meta[kMaxTapeIters];  // and their counts
    float4* p_fin;                 // with viscosity: the frame's final positions and the
    float4* v_u;                   // velocities before the viscosity pass (sorted order)
    float* w;                      // with solids: the inverse masses (sorted order)
    float4* omega;                 // with vorticity: the frame's omega and eta (sorted order) and
    float4* eta;
    float4* fext;                  // the external force its applyForces took (pre-sort order)
    uint32_t* full;                // with viscosity or vorticity: the frame's full list (recorded
    uint32_t* full_meta;           // here instead of the simulation's buffer; stride N)
};

struct pbd_sim {
    pbd_params prm{};
    uint32_t cap = 0, N = 0;
    int device = 0, num_sms = 0;
    void* arena = nullptr;
    float4 *x[2]{}, *p[3]{}, *v[2]{}, *col[2]{};
    uint32_t* ids[2]{};
    float* w[2]{};                // inverse masses (solids = 0), carried through re-orders once used
    bool mass_used = false;
    int tpb_nbr = kThreadsNeighbourDefault;   // block size of the neighbour passes (tunable)
    // batched form
    bool batched = false;
    uint32_t nscenes = 0;
    SceneParams* d_scenes = nullptr;
    uint32_t* scene_of = nullptr;
    uint32_t* scene_range = nullptr;
    // adjoint workspace (allocated by pbd_adjoint_forward)
    void* adj_arena = nullptr;
    size_t adj_bytes = 0;
    int adj_steps = 0, adj_every = 0, adj_nck = 0;
    uint32_t adj_n = 0;
    float4 *adj_ck_x = nullptr, *adj_ck_v = nullptr, *adj_fin_x = nullptr, *adj_fin_v = nullptr;
    uint32_t* adj_fin_keys = nullptr;
    float4 *adj_fin_p = nullptr, *adj_fin_col = nullptr;
    uint32_t* adj_fin_ids = nullptr;
    float *adj_ck_w = nullptr, *adj_fin_w = nullptr;   // with solids: the inverse masses (permuted with the state)
    float4 *adj_ck_f = nullptr, *adj_fin_f = nullptr;  // with vorticity: the force the next frame applies
    std::vector<Tape> adj_tape;
    float4 *adj_g[6]{};            // gradient buffers
    float* adj_glam = nullptr;
    unsigned long long* adj_scat3 = nullptr;  // with vorticity: partners' dL/domega terms, fixed point
    float4* adj_gom = nullptr;                // with vorticity: each particle's own dL/domega
    bool adj_last_taped = false;   // the tape holds the forward's last segment
    uint64_t gen = 0, adj_gen = 0; // bumped by every call that changes the state or parameters
    uint64_t pgen = 0;             // bumped by every call that changes the parameters, N or the block size
    int anchor = -1;               // p buffer holding the last frame's anchors (-1: none since the state changed)
    // collisionType 1 workspace (allocated when the parameters select it, never inside a frame)
    void* ct_arena = nullptr;
    size_t ct_bytes = 0;
    ContactStore ct{};
    // sprite image workspace (allocated by pbd_render_sprites on first use or growth)
    void* img_arena = nullptr;
    size_t img_bytes = 0;
    double* stats = nullptr;       // device accumulators of pbd_density_error
    struct AdjGraph { Cur start; int nf; int kind; Cur end; cudaGraphExec_t exec; };   // kind: see adj_segment
    std::vector<AdjGraph> adj_graphs;   // recorded segments of the adjoint
    uint64_t adj_graphs_pgen = ~0ull;
    void* adj_graphs_arena = nullptr;
    double* adj_acc = nullptr;               // per reverse block: dL/drest_density, dL/deps
    uint32_t* adj_gmax = nullptr;            // the frame's largest entering gradient (fixed-point scale)
    unsigned long long* adj_scat = nullptr;  // partners' terms of a delta reverse pass, fixed point (4 per particle)
    unsigned long long* adj_scat2 = nullptr; // the same for the lambda reverse passes
    std::vector<uint32_t> scene_cap, scene_count;
    std::vector<SceneParams> h_scenes;
    float4 *fext = nullptr, *omega = nullptr, *delta = nullptr;
    float* lambda = nullptr;
    uint32_t *keys[2]{}, *vals[2]{};
    uint32_t *cell_start = nullptr, *cell_end = nullptr;
    uint32_t *hist = nullptr, *status = nullptr, *tile_counter = nullptr, *err = nullptr, *table_n = nullptr;
    uint32_t max_tiles = 0;
    uint32_t *nb_list = nullptr, *nb_meta = nullptr;   // near lists (recorded by lambda / omega)
    uint32_t *fl_list = nullptr, *fl_meta = nullptr;   // full lists (recorded by the frame's first lambda)
    uint32_t *defer_items = nullptr, *defer_count = nullptr, *defer_done = nullptr;
    uint32_t defer_cap = 0;
    // particles without a stored list, walked by the leading blocks of the list passes:
    // DF = no full list (noted by the frame's first lambda pass), DN = no near list (noted by
    // the pass that records the near lists, emptied by the pass that reads them)
    uint32_t *dfr_items = nullptr, *dfr_count = nullptr, *dnr_items = nullptr, *dnr_count = nullptr;
    Cur cur;
    int table_passes = -1;        // passes of the sort whose keys the cell tables hold (-1: none)
    uint32_t table_hint = 0;      // host upper bound of the device word table_n
    cudaStream_t last_stream = nullptr;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t exec[kMaxGraphs]{};
    Cur exec_start[kMaxGraphs];
    Cur exec_end[kMaxGraphs];
    int nexec = 0;
    // pbd_step_readback: pinned host copies of x and v (2 x capacity float4, allocated on first
    // use; rb_dev is the same memory as the device addresses it), a side stream for the position
    // copy, and frame graphs (one per entry of exec) that copy the positions beside the frame's
    // omega / vorticity / viscosity passes
    float4* rb_host = nullptr;
    float4* rb_dev = nullptr;
    cudaStream_t rb_stream = nullptr;
    cudaEvent_t rb_fork = nullptr, rb_join = nullptr;
    cudaGraphExec_t rb_exec[kMaxGraphs]{};
    int rb_n = 0;
    uint32_t graph_n = 0xFFFFFFFFu;
    bool dirty = true;
    uint32_t launches = 0;
    uint32_t batch_cells = 0;                // batched form: cells of all scenes' slices
    uint32_t fl_slots = 0;                   // slots of the full list per particle
    uint32_t sort_spin_limit = kSpinLimit;   // pbd_debug_set_wait_limit
    uint32_t sort_hold = 0;
};

namespace {

int cuda_fail(const char* what, cudaError_t e) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return PBD_ERR_CUDA;
}
#define CK(call)                                         \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return cuda_fail(#call, _e); \
    } while (0)

int sort_passes(const pbd_sim* s) {
    // With applyForces on, every key comes from a position clamped inside the enclosure, whose
    // limits are at most 126.5 (Communication.h:573-598): keys < 2^21, three 8-bit digits.
    // The batched form prefixes the scene number: 21 + log2(scenes) bits.
    if (s->batched) {   // keys run up to the last scene's slice end
        uint32_t bits = 1;
        while (bits < 32 && (1ull << bits) < s->batch_cells) ++bits;
        return std::min(kMaxPasses, (int)((bits + kRadixBits - 1) / kRadixBits));
    }
    return (s->prm.active & PBD_ACTIVE_APPLY_FORCES) ? 3 : 4;
}

uint32_t host_expand_bits(uint32_t v) {   // Hash.h:10-16, for the scenes' table slices
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

uint32_t table_size(const pbd_sim* s) { return s->batched ? s->batch_cells : s->prm.max_grid; }

float powi_host(float x, int n) {
    float r = 1.0f;
    for (int k = 0; k < n; ++k) r *= x;
    return r;
}

DevParams make_dev_params(const pbd_sim* s) {
    const pbd_params& p = s->prm;
    DevParams P{};
    P.N = s->N;
    P.G = p.max_grid;
    P.M = p.max_neighbours_per_particle;
    P.K = p.kernel_width_neighbours;
    P.active = p.active;
    P.flags = p.flags;
    P.n_scorr = p.n_scorr;
    P.d = 2.0f * p.particle_radius;                       // Initialize.h:43
    P.dt = p.delta_t;
    P.inv_dt = 1.0f / p.delta_t;
    P.gravity = p.gravity;
    P.rho0 = p.rest_density;
    P.hs = P.d * p.kernel_width_spiky;                    // Initialize.h:45
    P.hp = p.kernel_width_poly;                           // Initialize.h:53
    P.hp2 = P.hp * P.hp;
    P.hp_lim = P.hp - 0.001f;
    P.k_scorr = p.k_scorr;
    P.c_visc = p.c_viscosity;
    P.e_vort = p.e_vorticity;
    P.stiffness = p.stiffness;
    P.one_minus_stiffness = 1.0f - p.stiffness;
    P.pos_damp = p.enclosure_position_damping;
    P.vel_damp = p.enclosure_velocity_damping;
    P.lambda_eps = p.lambda_epsilon;
    for (int a = 0; a < 3; ++a) { P.bmin[a] = p.bounds_min[a]; P.bmax[a] = p.bounds_max[a]; }
    const double kPi = 3.14159265359;                     // Globals.h:122
    P.poly_inv_den = (float)(1.0 / ((double)0.001f + 64.0 * kPi * (double)powi_host(P.hp, 9)));
    P.spiky_den = (float)(kPi * (double)powi_host(P.hs, 6));
    // s_corr reference value: poly6 at distance |q|, q = spiky width x qSCorr (Initialize.h:49)
    const float q = P.hs * p.q_scorr;
    const float qd = std::sqrt(q * q + 0.0f + 0.0f);
    float wq = 0.0f;
    if (qd > 0.001f && qd < P.hp - 0.001f) {
        float t = P.hp2 - qd * qd;
        float t3 = t * t * t;
        wq = (315.0f * t3 * t3) * P.poly_inv_den;
    }
    P.wq = wq;
    P.inv_wq = wq != 0.0f ? 1.0f / wq : 0.0f;
    P.inv_spiky_den = 1.0f / P.spiky_den;
    P.far_pairs_zero = (wq > 0.0f && std::isfinite(wq) && p.n_scorr >= 0) ? 1u : 0u;
    P.batched = s->batched ? 1u : 0u;
    P.nscenes = s->nscenes;
    P.table_size = table_size(s);
    P.scenes = s->d_scenes;
    P.scene_of = s->scene_of;
    P.scene_range = s->scene_range;
    P.eta_tape = nullptr;
    const float c = std::max(P.hp, std::max(P.hs, P.d));
    P.cut2 = c * c * 1.0001f;
    return P;
}

// Optional per-launch timing: a pair of events around every kernel of a frame.
struct Profiler {
    struct Rec { const char* name; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    cudaStream_t st = nullptr;
    const char* pending = nullptr;
    void begin(const char* name) {
        Rec r{name, nullptr, nullptr};
        cudaEventCreate(&r.a);
        cudaEventCreate(&r.b);
        cudaEventRecord(r.a, st);
        recs.push_back(r);
    }
    void end() { cudaEventRecord(recs.back().b, st); }
    ~Profiler() {
        for (auto& r : recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    }
};
#define PROF_BEGIN(name) do { if (prof) prof->begin(name); } while (0)
#define PROF_END() do { if (prof) prof->end(); } while (0)

// The frame's first lambda pass stores the full list (its walk of the anchor cells) for the
// passes after it.
static bool use_full_list(const pbd_sim* s) {
    return !(s->prm.flags & PBD_FLAG_FULL_WALK) && (s->prm.active & PBD_ACTIVE_COMPUTE_LAMBDA) &&
           s->prm.solver_iterations > 0;
}

// Near lists need kernels that vanish beyond the cut (far_pairs_zero), and they pay only when the
// cut keeps a small part of the list: the cut's sphere against the cube of cells the list covers.
// With kernel widths of a few cells (config.txt's 4.1 and 6.1 with kernelWidthNeighbours 2) the
// sphere holds the whole cube, every entry is near, and the passes read the full list instead.
static bool near_lists_on(const pbd_sim* s, const DevParams& P) {
    if ((s->prm.flags & PBD_FLAG_FULL_WALK) || P.far_pairs_zero == 0u) return false;
    const bool shells = (P.active & PBD_ACTIVE_FIND_NEIGHBOURS) && P.K > 1;
    const double side = (2.0 * (shells ? P.K : 1u) + 1.0) * P.d;
    const double cut = std::sqrt((double)P.cut2 / 1.0001);
    return (4.0 / 3.0) * 3.14159265358979 * cut * cut * cut < 0.5 * side * side * side;
}

// delta_staged_kernel for `mode`, as launch_delta_list.
static void launch_delta_staged(uint32_t N, cudaStream_t st, const DevParams& P, uint32_t mode, const float4* pin,
                                const float4* pa, float4* pout, float4* x, float4* v, const float* lam, const float* w,
                                float4* delta, const uint32_t* cs, const uint32_t* ce, const CoopSet& C, const NbList& F) {
    constexpr uint32_t kFluid = kDoDelta | kDoCollide | kDoApply;
    const uint32_t g = C.blocks + (N + kStageThreads - 1) / kStageThreads;
    if (mode == kFluid)
        delta_staged_kernel<kFluid><<<g, kStageThreads, 0, st>>>(P, mode, pin, pa, pout, x, v, lam, w, delta, cs, ce, C, F);
    else if (mode == (kFluid | kDoUpdate))
        delta_staged_kernel<kFluid | kDoUpdate><<<g, kStageThreads, 0, st>>>(P, mode, pin, pa, pout, x, v, lam, w, delta, cs, ce, C, F);
    else
        delta_staged_kernel<0><<<g, kStageThreads, 0, st>>>(P, mode, pin, pa, pout, x, v, lam, w, delta, cs, ce, C, F);
}

// delta_list_kernel for `mode`: the fluid frame's two pass modes run specialised code.
static void launch_delta_list(uint32_t gn, int tn, cudaStream_t st, const DevParams& P, uint32_t mode,
                              const float4* pin, const float4* pa, float4* pout, float4* x, float4* v, const float* lam,
                              const float* w, float4* delta, const uint32_t* cs, const uint32_t* ce, const CoopSet& C,
                              const NbList& L, bool full) {
    constexpr uint32_t kFluid = kDoDelta | kDoCollide | kDoApply;
    const uint32_t g = gn + C.blocks;
    if (full) {   // the frame's full list: entries in batches of kListBatch
        if (mode == kFluid)
            delta_list_kernel<kFluid, kListBatch><<<g, tn, 0, st>>>(P, mode, pin, pa, pout, x, v, lam, w, delta, cs, ce, C, L);
        else if (mode == (kFluid | kDoUpdate))
            delta_list_kernel<kFluid | kDoUpdate, kListBatch><<<g, tn, 0, st>>>(P, mode, pin, pa, pout, x, v, lam, w, delta, cs, ce, C, L);
        else
            delta_list_kernel<0, kListBatch><<<g, tn, 0, st>>>(P, mode, pin, pa, pout, x, v, lam, w, delta, cs, ce, C, L);
        return;
    }
    if (mode == kFluid)
        delta_list_kernel<kFluid><<<g, tn, 0, st>>>(P, mode, pin, pa, pout, x, v, lam, w, delta, cs, ce, C, L);
    else if (mode == (kFluid | kDoUpdate))
        delta_list_kernel<kFluid | kDoUpdate><<<g, tn, 0, st>>>(P, mode, pin, pa, pout, x, v, lam, w, delta, cs, ce, C, L);
    else
        delta_list_kernel<0><<<g, tn, 0, st>>>(P, mode, pin, pa, pout, x, v, lam, w, delta, cs, ce, C, L);
}

// Record (or run) one frame of Fluid::compute (Fluid.cu:14-97) on `st`.
// readback: copy the final positions to s->rb_host on s->rb_stream once they are final (beside
// the frame's remaining passes); the final velocities go with them when viscosity does not
// change them, else the viscosity pass over the lists stores them into s->rb_host itself (other
// paths copy them at the end of the frame).
cudaError_t enqueue_frame(pbd_sim* s, cudaStream_t st, Cur& cur, bool front_only, uint32_t& nl,
                          Profiler* prof = nullptr, const Tape* tape = nullptr, bool readback = false) {
    DevParams P = make_dev_params(s);
    if (tape) P.eta_tape = tape->eta;   // a taped frame keeps the vorticity pass's eta
    const pbd_params& prm = s->prm;
    const uint32_t N = s->N;
    const int np = sort_passes(s);
    const int tn = s->tpb_nbr;
    SortScratch S{s->hist, s->status, s->tile_counter, s->err, s->max_tiles, s->sort_spin_limit, s->sort_hold};
    nl = 0;

    // applyForces + initializeCellIds (+ histograms, + clearing last frame's cells)
    const uint32_t total = std::max(N, s->table_hint);
    const uint32_t gpred = std::max(1u, std::min(div_up(total, kThreadsParticle), (uint32_t)s->num_sms * 8u));
    if (tape) {
        cudaMemcpyAsync(tape->x_in, s->x[cur.x], (size_t)N * 16, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(tape->v_in, s->v[cur.v], (size_t)N * 16, cudaMemcpyDeviceToDevice, st);
        if (tape->fext) cudaMemcpyAsync(tape->fext, s->fext, (size_t)N * 16, cudaMemcpyDeviceToDevice, st);
    }
    PROF_BEGIN("predict_key");
    const float* wcur = s->mass_used ? s->w[cur.x] : nullptr;
    predict_key_kernel<<<gpred, kThreadsParticle, 0, st>>>(P, s->x[cur.x], s->v[cur.v], s->p[cur.p], s->fext, wcur,
                                                           s->keys[0], s->keys[np % 2], s->table_n, s->cell_start,
                                                           s->hist, np, s->err, s->dfr_count);
    PROF_END();
    ++nl;
    // sortIds
    const uint32_t ntiles = div_up(N, kSortTile);
    for (int pass = 0; pass < np; ++pass) {
        const int in = pass % 2, out = (pass + 1) % 2;
        PROF_BEGIN("onesweep_pass");
        if (pass == 0)
            onesweep_pass<true><<<ntiles, kSortThreads, 0, st>>>(s->keys[in], s->vals[in], s->keys[out], s->vals[out], N, pass, S);
        else
            onesweep_pass<false><<<ntiles, kSortThreads, 0, st>>>(s->keys[in], s->vals[in], s->keys[out], s->vals[out], N, pass, S);
        PROF_END();
        ++nl;
    }
    // copy + reorder + computeCellInfo
    const int fin = np % 2;
    if (tape) {
        cudaMemcpyAsync(tape->perm, s->vals[fin], (size_t)N * 4, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(tape->keys, s->keys[fin], (size_t)N * 4, cudaMemcpyDeviceToDevice, st);
    }
    const bool cols = (prm.flags & PBD_FLAG_COLORS) != 0, ids = (prm.flags & PBD_FLAG_TRACK_IDS) != 0;
    const int anchor = (cur.p + 1) % 3;   // this frame's anchor: never written again in the frame
    ReorderArgs A{s->keys[fin], s->vals[fin], s->x[cur.x], s->p[cur.p], s->v[cur.v], s->col[cur.x],
                  s->x[cur.x ^ 1], s->p[anchor], s->v[cur.v ^ 1], cols ? s->col[cur.x ^ 1] : nullptr,
                  s->ids[cur.x], ids ? s->ids[cur.x ^ 1] : nullptr, s->w[cur.x], s->mass_used ? s->w[cur.x ^ 1] : nullptr,
                  s->cell_start, s->cell_end, s->table_n};
    const uint32_t greo = std::max(div_up(N, kThreadsParticle), div_up((uint64_t)ntiles * kRadix, kThreadsParticle));
    PROF_BEGIN("reorder_cells");
    reorder_cells_kernel<<<std::max(1u, greo), kThreadsParticle, 0, st>>>(P, A, S, np, ntiles);
    PROF_END();
    ++nl;
    cur.x ^= 1; cur.p = anchor; cur.v ^= 1;
    if (front_only) return cudaGetLastError();
    const float4* pa = s->p[anchor];
    const float* wf = s->mass_used ? s->w[cur.x] : nullptr;   // after the re-order
    if (tape && tape->w && wf) cudaMemcpyAsync(tape->w, wf, (size_t)N * 4, cudaMemcpyDeviceToDevice, st);
    auto next_p = [&](int c) { return c == anchor ? (anchor + 1) % 3 : 3 - c - anchor; };

    const uint32_t gn = div_up(N, tn);
    const DeferList D{s->defer_items, s->defer_count, s->defer_done, s->defer_cap};
    const uint32_t gc = (uint32_t)s->num_sms * 2u;   // cooperative kernels: grid-stride over the deferred
    // the list passes' own cooperative blocks: DF is read by every full-list pass of the frame,
    // DN emptied by the pass that reads it
    const DeferList DF{s->dfr_items, s->dfr_count, s->dfr_count + 1, s->defer_cap};
    const DeferList DN{s->dnr_items, s->dnr_count, s->dnr_count + 1, s->defer_cap};
    const DeferList DX{nullptr, nullptr, nullptr, 0u};
    const CoopSet CF{s->dfr_items, s->dfr_count, s->dfr_count + 1, s->defer_cap, kCoopBlocks, 0u};
    const CoopSet CN{s->dnr_items, s->dnr_count, s->dnr_count + 1, s->defer_cap, kCoopBlocks, 1u};
    const uint32_t act = prm.active;
    const uint32_t I = prm.solver_iterations, Sx = prm.stabilization_iterations;
    // near lists: recorded by a walking pass for the pass after it at the same positions; they
    // need kernels that vanish beyond the cut (far_pairs_zero)
    const bool use_lists = near_lists_on(s, P) && !(prm.flags & PBD_FLAG_STAGED_PASSES);
    const NbList Lf = use_lists ? NbList{s->nb_list, s->nb_meta, s->cap, kListMax} : NbList{nullptr, nullptr, 0u, 0u};
    const NbList L = Lf;
    const NbList L0{nullptr, nullptr, 0u, 0u};
    // full lists: stored by the first lambda pass of the frame (its walk of the anchor cells)
    const bool use_full = use_full_list(s);
    const NbList F = !use_full ? L0
                     : (tape && tape->full) ? NbList{tape->full, tape->full_meta, N, s->fl_slots}
                                            : NbList{s->fl_list, s->fl_meta, s->cap, s->fl_slots};
    // PBD_FLAG_STAGED_PASSES: the later lambda passes and the delta passes stage each block's
    // neighbourhood in shared memory (the full list stays the fallback); inverse masses are not
    // staged, so simulations with solids read the lists
    const bool staged_ok = (prm.flags & PBD_FLAG_STAGED_PASSES) && use_full && !use_lists && staged_supported(P) &&
                           !s->mass_used;
    const bool do_delta = act & PBD_ACTIVE_COMPUTE_DELTA_POSITIONS, do_apply = act & PBD_ACTIVE_APPLY_DELTA_POSITIONS;
    const bool do_update = act & PBD_ACTIVE_UPDATE_POSITIONS;
    const bool collide = prm.collision_type == 0;
    const bool batched_contacts = prm.collision_type == 1;
    if (batched_contacts) {   // every list entry of the frame is a constraint (Fluid.cu:37-47)
        PROF_BEGIN("contact_list");
        cudaMemsetAsync(s->ct.long_count, 0, 4, st);
        contact_list_kernel<<<div_up(N, kThreadsParticle), kThreadsParticle, 0, st>>>(P, pa, s->cell_start, s->cell_end, s->ct);
        PROF_END();
        ++nl;
        cudaMemsetAsync(s->ct.best, 0, (size_t)N * 8, st);   // the frame's first batch's keys
    }
    uint32_t nbatch = 0;   // contact batches so far in this frame: their keys alternate buffers
    bool last_was_delta = false;
    for (uint32_t it = 0; it < I; ++it) {
        if (tape && it < (uint32_t)kMaxTapeIters)
            cudaMemcpyAsync(tape->p_it[it], s->p[cur.p], (size_t)N * 16, cudaMemcpyDeviceToDevice, st);
        // a taped frame keeps each iteration's lambda (and the sums behind it) for the reverse pass
        const bool taped = tape && it < (uint32_t)kMaxTapeIters;
        float* lam = taped ? tape->lam[it] : s->lambda;
        float4* aux = taped ? tape->aux[it] : nullptr;
        // a taped frame records the iteration's near lists into the tape (the delta pass reads them there)
        const NbList L = (taped && use_lists) ? NbList{tape->near[it], tape->near_meta[it], N, kListMax} : Lf;
        if (act & PBD_ACTIVE_COMPUTE_LAMBDA) {
            const bool lstaged = staged_ok && it > 0 && !aux;
            PROF_BEGIN(lstaged ? "lambda_staged" : ((use_full && it > 0) ? "lambda_list" : "lambda"));
            const NbList Lr = (act & PBD_ACTIVE_COMPUTE_DELTA_POSITIONS) ? L : L0;
            if (lstaged) {
                lambda_staged_kernel<<<kCoopBlocks + div_up(N, kStageThreads), kStageThreads, 0, st>>>(
                    P, s->p[cur.p], pa, s->cell_start, s->cell_end, lam, CF, F);
                nl += 1;
            } else if (use_full && it > 0) {
                lambda_list_kernel<<<gn + kCoopBlocks, tn, 0, st>>>(P, s->p[cur.p], pa, s->cell_start, s->cell_end, lam,
                                                                    CF, Lr.list ? DN : DX, aux, Lr, F);
                nl += 1;
            } else {
                lambda_kernel<<<gn, tn, 0, st>>>(P, s->p[cur.p], pa, s->cell_start, s->cell_end, lam, D, aux, Lr,
                                                 use_full ? F : L0, use_full ? DF : DX, Lr.list ? DN : DX);
                lambda_coop_kernel<<<gc, kThreadsCoop, 0, st>>>(P, s->p[cur.p], pa, s->cell_start, s->cell_end, lam, D, aux);
                nl += 2;
            }
            PROF_END();
            last_was_delta = false;
        }
        if (batched_contacts) {
            // collisionType 1 (Fluid.cu:55-77): delta positions, then S passes of contact
            // batches on p* and x in place, then applyDeltaPositions (+ updatePositions)
            const bool recorded = (act & PBD_ACTIVE_COMPUTE_LAMBDA) && (act & PBD_ACTIVE_COMPUTE_DELTA_POSITIONS);
            if (do_delta) {
                const uint32_t mode = kDoDelta | kStoreDelta;
                const bool by_list = use_lists ? recorded : use_full;
                PROF_BEGIN(by_list ? "delta_list" : "delta");
                const int pout = next_p(cur.p);
                if (by_list) {
                    launch_delta_list(gn, tn, st, P, mode, s->p[cur.p], pa, s->p[pout], s->x[cur.x], s->v[cur.v], lam, wf,
                                      s->delta, s->cell_start, s->cell_end, use_lists ? CN : CF, use_lists ? L : F, !use_lists);
                    nl += 1;
                } else {
                    delta_kernel<<<gn, tn, 0, st>>>(P, mode, s->p[cur.p], pa, s->p[pout], s->x[cur.x], s->v[cur.v], lam, wf,
                                                    s->delta, s->cell_start, s->cell_end, D);
                    delta_coop_kernel<<<gc, kThreadsCoop, 0, st>>>(P, mode, s->p[cur.p], pa, s->p[pout], s->x[cur.x],
                                                                   s->v[cur.v], lam, wf, s->delta, s->cell_start, s->cell_end, D);
                    nl += 2;
                }
                PROF_END();
                cur.p = pout;
            }
            // the batches' keys alternate between two buffers; each solve pass clears the other
            ContactStore C = s->ct;
            unsigned long long* const keys[2] = {s->ct.best, s->ct.best + s->ct.stride};
            const size_t words = (C.M + 31) / 32;
            for (uint32_t k = 0; k < Sx; ++k) {
                PROF_BEGIN("contact_batches");
                cudaMemsetAsync(C.solved, 0, words * C.stride * 4, st);
                for (uint32_t b = 0; b < prm.max_collision_batches; ++b, ++nbatch) {
                    C.best = keys[nbatch & 1u];
                    C.best_next = keys[(nbatch + 1u) & 1u];
                    contact_claim_kernel<<<kClaimCoopBlocks + div_up(N, kThreadsParticle / kClaimLanes), kThreadsParticle, 0, st>>>(P, C, s->p[cur.p], wf);
                    contact_solve_kernel<<<div_up(N, kThreadsParticle), kThreadsParticle, 0, st>>>(P, C, s->p[cur.p], s->x[cur.x], wf);
                    nl += 2;
                }
                PROF_END();
            }
            uint32_t mode = 0;
            if (do_apply) mode |= kLoadDelta | kDoApply;
            if (it + 1 == I && do_update && mode) mode |= kDoUpdate;
            if (mode) {
                PROF_BEGIN("apply");
                const int pout = next_p(cur.p);
                delta_kernel<<<gn, tn, 0, st>>>(P, mode, s->p[cur.p], pa, s->p[pout], s->x[cur.x], s->v[cur.v], lam, wf,
                                                s->delta, s->cell_start, s->cell_end, D);
                PROF_END();
                ++nl;
                cur.p = pout;
                last_was_delta = (mode & kDoUpdate) != 0;
            }
            continue;
        }
        // passes of this iteration: pass 0 carries computeDeltaPositions and the first
        // solveCollisions; pass k carries solveCollisions k; applyDeltaPositions rides on the
        // last pass.
        const uint32_t ncoll = collide ? Sx : 0u;
        const uint32_t npass = std::max(1u, ncoll);
        for (uint32_t k = 0; k < npass; ++k) {
            uint32_t mode = 0;
            if (k == 0 && do_delta) mode |= kDoDelta;
            if (k < ncoll) mode |= kDoCollide;
            const bool last = (k + 1 == npass);
            if (last && do_apply) {
                mode |= kDoApply;
                if (!(mode & kDoDelta)) mode |= kLoadDelta;
            }
            if ((mode & kDoDelta) && (!last || !do_apply)) mode |= kStoreDelta;
            if (mode == 0) continue;
            // a taped frame keeps the positions a later contact pass starts from
            if (taped && k >= 1 && k < (uint32_t)kMaxTapeStab && tape->p_s[it][k - 1])
                cudaMemcpyAsync(tape->p_s[it][k - 1], s->p[cur.p], (size_t)N * 16, cudaMemcpyDeviceToDevice, st);
            const bool final_pass = last && (it + 1 == I);
            if (final_pass && do_update) mode |= kDoUpdate;
            const bool recorded = (act & PBD_ACTIVE_COMPUTE_LAMBDA) && (act & PBD_ACTIVE_COMPUTE_DELTA_POSITIONS);
            // the near lists hold this iteration's lambda walk (same positions) on pass 0 only;
            // without near lists every pass reads the frame's full list
            const bool by_list = use_lists ? (k == 0 && recorded) : use_full;
            const bool dstaged = by_list && staged_ok && !taped;
            PROF_BEGIN(dstaged ? "delta_staged" : (by_list ? "delta_list" : "delta"));
            const int pout = next_p(cur.p);
            if (dstaged) {
                launch_delta_staged(N, st, P, mode, s->p[cur.p], pa, s->p[pout], s->x[cur.x], s->v[cur.v], lam, wf,
                                    s->delta, s->cell_start, s->cell_end, CF, F);
                nl += 1;
            } else if (by_list) {
                launch_delta_list(gn, tn, st, P, mode, s->p[cur.p], pa, s->p[pout], s->x[cur.x], s->v[cur.v], lam, wf,
                                  s->delta, s->cell_start, s->cell_end, use_lists ? CN : CF, use_lists ? L : F, !use_lists);
                nl += 1;
            } else {
                delta_kernel<<<gn, tn, 0, st>>>(P, mode, s->p[cur.p], pa, s->p[pout], s->x[cur.x], s->v[cur.v], lam, wf,
                                                s->delta, s->cell_start, s->cell_end, D);
                delta_coop_kernel<<<gc, kThreadsCoop, 0, st>>>(P, mode, s->p[cur.p], pa, s->p[pout], s->x[cur.x],
                                                               s->v[cur.v], lam, wf, s->delta, s->cell_start, s->cell_end, D);
                nl += 2;
            }
            PROF_END();
            cur.p = pout;
            last_was_delta = (mode & kDoUpdate) != 0;
        }
    }
    if (do_update && !last_was_delta) {
        PROF_BEGIN("update");
        update_kernel<<<div_up(N, kThreadsParticle), kThreadsParticle, 0, st>>>(P, s->p[cur.p], s->x[cur.x], s->v[cur.v]);
        PROF_END();
        ++nl;
    }
    const int vort = (act & PBD_ACTIVE_COMPUTE_VORTICITY) != 0, visc = (act & PBD_ACTIVE_COMPUTE_VISCOSITY) != 0;
    if (tape && (visc || vort) && tape->p_fin) {   // what the viscosity's and vorticity's reverse passes read
        cudaMemcpyAsync(tape->p_fin, s->x[cur.x], (size_t)N * 16, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(tape->v_u, s->v[cur.v], (size_t)N * 16, cudaMemcpyDeviceToDevice, st);
    }
    bool v_read = false;   // the frame's final velocities are on their way to s->rb_host
    if (readback) {   // x (and v, unless viscosity follows) is final: copy it while the last passes run
        cudaEventRecord(s->rb_fork, st);
        cudaStreamWaitEvent(s->rb_stream, s->rb_fork, 0);
        cudaMemcpyAsync(s->rb_host, s->x[cur.x], (size_t)N * 16, cudaMemcpyDeviceToHost, s->rb_stream);
        if (!visc) {
            cudaMemcpyAsync(s->rb_host + s->cap, s->v[cur.v], (size_t)N * 16, cudaMemcpyDeviceToHost, s->rb_stream);
            v_read = true;
        }
        cudaEventRecord(s->rb_join, s->rb_stream);
    }
    if (act & PBD_ACTIVE_COMPUTE_OMEGAS) {
        PROF_BEGIN(use_full ? "omega_list" : "omega");
        // near lists for viscosity: read by viscosity alone, or beside the full list for vorticity
        // (omega filters them out of the full list before its sums)
        const NbList Lo = ((vort || visc) && (use_full || !vort)) ? L : L0;
        // viscosity alone walks them: the particles left without one go to its cooperative blocks
        const DeferList DNo = (Lo.list && !vort) ? DN : DX;
        if (use_full) {
            if (Lo.list)
                omega_list_kernel<true><<<gn + kCoopBlocks, tn, 0, st>>>(P, s->p[cur.p], pa, s->v[cur.v], s->cell_start, s->cell_end,
                                                               s->omega, CF, DNo, Lo, F);
            else
                omega_list_kernel<false><<<gn + kCoopBlocks, tn, 0, st>>>(P, s->p[cur.p], pa, s->v[cur.v], s->cell_start, s->cell_end,
                                                               s->omega, CF, DNo, Lo, F);
            nl += 1;
        } else {
            omega_kernel<<<gn, tn, 0, st>>>(P, s->p[cur.p], pa, s->v[cur.v], s->cell_start, s->cell_end, s->omega, D, Lo, DNo);
            omega_coop_kernel<<<gc, kThreadsCoop, 0, st>>>(P, s->p[cur.p], pa, s->v[cur.v], s->cell_start, s->cell_end, s->omega, D);
            nl += 2;
        }
        PROF_END();
        if (tape && tape->omega) cudaMemcpyAsync(tape->omega, s->omega, (size_t)N * 16, cudaMemcpyDeviceToDevice, st);
    }
    if (vort || visc) {
        // vorticity sums every list entry: the full list; viscosity alone: the omega pass's near list
        // (without near lists, viscosity alone reads the full list too)
        const bool vfull = vort || (!use_lists && use_full);
        const NbList Lv = vfull ? F : ((act & PBD_ACTIVE_COMPUTE_OMEGAS) ? L : L0);
        const NbList Ln = (vort && use_full && (act & PBD_ACTIVE_COMPUTE_OMEGAS)) ? L : L0;
        PROF_BEGIN(Lv.list ? "vort_visc_list" : "vort_visc");
        if (Lv.list) {
            float4* const vh = (readback && visc) ? s->rb_dev + s->cap : nullptr;
            if (Ln.list)
                vort_visc_list_kernel<true><<<gn + kCoopBlocks, tn, 0, st>>>(P, s->p[cur.p], pa, s->v[cur.v], s->v[cur.v ^ 1], s->omega,
                                                                   s->fext, s->cell_start, s->cell_end, vort, visc, wf,
                                                                   vfull ? CF : CN, Lv, Ln, vh);
            else
                vort_visc_list_kernel<false><<<gn + kCoopBlocks, tn, 0, st>>>(P, s->p[cur.p], pa, s->v[cur.v], s->v[cur.v ^ 1], s->omega,
                                                                   s->fext, s->cell_start, s->cell_end, vort, visc, wf,
                                                                   vfull ? CF : CN, Lv, Ln, vh);
            v_read = v_read || vh != nullptr;
            nl += 1;
        } else {
            vort_visc_kernel<<<gn, tn, 0, st>>>(P, s->p[cur.p], pa, s->v[cur.v], s->v[cur.v ^ 1], s->omega, s->fext,
                                                s->cell_start, s->cell_end, vort, visc, wf, D);
            vort_visc_coop_kernel<<<gc, kThreadsCoop, 0, st>>>(P, s->p[cur.p], pa, s->v[cur.v], s->v[cur.v ^ 1], s->omega,
                                                               s->fext, s->cell_start, s->cell_end, vort, visc, wf, D);
            nl += 2;
        }
        PROF_END();
        if (visc) cur.v ^= 1;
    }
    if (readback) {
        if (!v_read) cudaMemcpyAsync(s->rb_host + s->cap, s->v[cur.v], (size_t)N * 16, cudaMemcpyDeviceToHost, st);
        cudaStreamWaitEvent(st, s->rb_join, 0);
    }
    return cudaGetLastError();
}

void destroy_graphs(pbd_sim* s) {
    for (int k = 0; k < kMaxGraphs; ++k) {
        if (s->exec[k]) { cudaGraphExecDestroy(s->exec[k]); s->exec[k] = nullptr; }
        if (s->rb_exec[k]) { cudaGraphExecDestroy(s->rb_exec[k]); s->rb_exec[k] = nullptr; }
    }
    s->nexec = 0;
    s->rb_n = 0;
}

int capture_one(pbd_sim* s, Cur& c, cudaGraphExec_t* out, uint32_t& nl, bool readback = false) {
    CK(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_frame(s, s->cap_stream, c, false, nl, nullptr, nullptr, readback);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(s->cap_stream, &g);
    if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail("frame capture", e); }
    if (e2 != cudaSuccess) return cuda_fail("cudaStreamEndCapture", e2);
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail("cudaGraphInstantiate", e);
    return PBD_OK;
}

// The sort's final buffer depends on the pass count; if it moved, clear the old cells now.
int settle_tables(pbd_sim* s, cudaStream_t st) {
    const int np = sort_passes(s);
    if (s->table_passes >= 0 && (s->table_passes % 2) != (np % 2)) {
        clear_cells_kernel<<<std::max(1u, std::min(div_up(s->table_hint, 256), (uint32_t)s->num_sms * 8u)), 256, 0, st>>>(
            s->keys[s->table_passes % 2], s->table_n, s->cell_start, table_size(s));
        CK(cudaGetLastError());
        CK(cudaMemsetAsync(s->table_n, 0, sizeof(uint32_t), st));
        s->table_hint = 0;
    }
    s->table_passes = np;
    return PBD_OK;
}

int build_graphs(pbd_sim* s) {
    destroy_graphs(s);
    Cur c = s->cur;
    uint32_t nl = 0;
    // follow the cycle of starting records: frame k starts where frame k-1 ended
    for (int k = 0; k < kMaxGraphs; ++k) {
        const Cur start = c;
        int rc = capture_one(s, c, &s->exec[k], nl);
        if (rc) return rc;
        s->exec_start[k] = start;
        s->exec_end[k] = c;
        s->nexec = k + 1;
        bool closed = false;
        for (int j = 0; j <= k; ++j) closed = closed || (s->exec_start[j] == c);
        if (closed) {
            s->launches = nl;
            s->graph_n = s->N;
            s->dirty = false;
            return PBD_OK;
        }
    }
    set_error("internal: the frame's buffer records do not cycle");
    return PBD_ERR_CUDA;
}

// The readback twin of every recorded frame graph (same start and end records).
int build_rb_graphs(pbd_sim* s) {
    for (int k = 0; k < s->nexec; ++k) {
        Cur c = s->exec_start[k];
        uint32_t nl = 0;
        if (int rc = capture_one(s, c, &s->rb_exec[k], nl, true)) return rc;
        if (!(c == s->exec_end[k])) { set_error("internal: readback frame ends elsewhere"); return PBD_ERR_CUDA; }
    }
    s->rb_n = s->nexec;
    return PBD_OK;
}

int check_sim(const pbd_sim* s, const char* fn) {
    if (!s) { set_error(std::string(fn) + ": null handle"); return PBD_ERR_INVALID_ARG; }
    return PBD_OK;
}

int sync_last(pbd_sim* s) {
    CK(cudaStreamSynchronize(s->last_stream));
    return PBD_OK;
}

}  // namespace

// ======================================================================================
// C ABI
// ======================================================================================
extern "C" {

const char* pbd_last_error(void) { return g_last_error.c_str(); }
uint32_t pbd_abi_version(void) { return PBD_ABI_VERSION; }

}  // extern "C"

namespace {
// collisionType 1 keeps every list entry of the frame (up to M per particle) as a constraint:
// allocate that workspace when the parameters select it (at pbd_create / pbd_set_params).
int ensure_contacts(pbd_sim* s) {
    if (s->prm.collision_type != 1) return PBD_OK;
    const size_t C = s->cap, M = std::max(1u, s->prm.max_neighbours_per_particle), W = (M + 31) / 32;
    if (C * M >= (size_t(1) << 32)) {   // constraint indices are 32-bit
        set_error("collisionType 1: capacity x maxNeighboursPerParticle must stay below 2^32");
        return PBD_ERR_UNSUPPORTED;
    }
    const size_t need = ((C * M * 4 + 255) & ~size_t(255)) + ((C * 4 + 255) & ~size_t(255)) +
                        ((C * W * 4 + 255) & ~size_t(255)) + C * 16 + ((C * 4 + 255) & ~size_t(255)) + 256 + 256;
    if (s->ct_arena && s->ct_bytes >= need && s->ct.M == M) return PBD_OK;
    if (s->ct_arena) {
        cudaDeviceSynchronize();
        cudaFree(s->ct_arena);
        s->ct_arena = nullptr;
        s->ct_bytes = 0;
    }
    cudaError_t e = lib_malloc(&s->ct_arena, need);
    if (e != cudaSuccess) { set_error(std::string("collisionType 1 workspace: ") + cudaGetErrorString(e)); return PBD_ERR_ALLOC; }
    s->ct_bytes = need;
    char* c = static_cast<char*>(s->ct_arena);
    auto take = [&](size_t b) { char* r = c; c += (b + 255) & ~size_t(255); return r; };
    s->ct.list = (uint32_t*)take(C * M * 4);
    s->ct.count = (uint32_t*)take(C * 4);
    s->ct.solved = (uint32_t*)take(C * W * 4);
    s->ct.best = (unsigned long long*)take(C * 16);   // two buffers of C keys
    s->ct.best_next = s->ct.best + C;
    s->ct.long_items = (uint32_t*)take(C * 4);
    s->ct.long_count = (uint32_t*)take(4);
    s->ct.stride = (uint32_t)C;
    s->ct.M = (uint32_t)M;
    return PBD_OK;
}

// Allocate a simulation: one arena for every buffer.  `scenes` is non-null for the batched form.
int create_sim(const pbd_params* prm, uint32_t capacity, const std::vector<SceneParams>* scenes,
               const std::vector<uint32_t>* caps, pbd_sim** out) {
    *out = nullptr;
    int rc = pbd_validate_params(prm);
    if (rc) return rc;
    if (capacity == 0 || capacity > (1u << 30) - 1u) { set_error("capacity must be in [1, 2^30)"); return PBD_ERR_INVALID_ARG; }
    pbd_sim* s = new (std::nothrow) pbd_sim();
    if (!s) { set_error("host allocation"); return PBD_ERR_ALLOC; }
    s->prm = *prm;
    s->cap = capacity;
    if (scenes) {
        s->batched = true;
        s->nscenes = (uint32_t)scenes->size();
        s->h_scenes = *scenes;
        s->batch_cells = scenes->back().base + scenes->back().cells;
        s->scene_cap = *caps;
        s->scene_count.assign(s->nscenes, 0u);
    }
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) { delete s; return cuda_fail("cudaGetDevice", e); }
    e = cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->device);
    if (e != cudaSuccess) { delete s; return cuda_fail("cudaDeviceGetAttribute", e); }
    s->max_tiles = div_up(capacity, kSortTile);
    // ---- one arena, 256-byte aligned slices
    const size_t C = capacity, T = table_size(s);
    std::vector<std::pair<void**, size_t>> parts;
    for (int b = 0; b < 2; ++b) {
        parts.push_back({(void**)&s->x[b], C * 16});
        parts.push_back({(void**)&s->v[b], C * 16}); parts.push_back({(void**)&s->col[b], C * 16});
        parts.push_back({(void**)&s->ids[b], C * 4}); parts.push_back({(void**)&s->w[b], C * 4});
        parts.push_back({(void**)&s->keys[b], C * 4}); parts.push_back({(void**)&s->vals[b], C * 4});
    }
    for (int b = 0; b < 3; ++b) parts.push_back({(void**)&s->p[b], C * 16});
    parts.push_back({(void**)&s->fext, C * 16}); parts.push_back({(void**)&s->omega, C * 16});
    parts.push_back({(void**)&s->delta, C * 16}); parts.push_back({(void**)&s->lambda, C * 4});
    parts.push_back({(void**)&s->cell_start, T * 4}); parts.push_back({(void**)&s->cell_end, T * 4});
    parts.push_back({(void**)&s->hist, (size_t)kMaxPasses * kRadix * 4});
    parts.push_back({(void**)&s->status, (size_t)kMaxPasses * s->max_tiles * kRadix * 4});
    parts.push_back({(void**)&s->tile_counter, kMaxPasses * 4}); parts.push_back({(void**)&s->err, 4});
    parts.push_back({(void**)&s->table_n, 4}); parts.push_back({(void**)&s->stats, 64});
    s->defer_cap = capacity;   // every particle can be handed to the cooperative kernels
    parts.push_back({(void**)&s->defer_items, (size_t)s->defer_cap * 4});
    parts.push_back({(void**)&s->defer_count, 4}); parts.push_back({(void**)&s->defer_done, 4});
    parts.push_back({(void**)&s->dfr_items, (size_t)s->defer_cap * 4}); parts.push_back({(void**)&s->dfr_count, 8});
    parts.push_back({(void**)&s->dnr_items, (size_t)s->defer_cap * 4}); parts.push_back({(void**)&s->dnr_count, 8});
    parts.push_back({(void**)&s->nb_list, (size_t)kListMax * C * 4}); parts.push_back({(void**)&s->nb_meta, C * 4});
    // full-list slots: kFullMax when the parameters reach beyond the 27 cells (shells), else
    // kFullSlim; longer lists are walked by a warp per particle instead (correct, slower)
    s->fl_slots = ((prm->active & PBD_ACTIVE_FIND_NEIGHBOURS) && prm->kernel_width_neighbours >= 2) ? kFullMax : kFullSlim;
    parts.push_back({(void**)&s->fl_list, (size_t)s->fl_slots * C * 4}); parts.push_back({(void**)&s->fl_meta, C * 4});
    if (s->batched) {
        parts.push_back({(void**)&s->d_scenes, (size_t)s->nscenes * sizeof(SceneParams)});
        parts.push_back({(void**)&s->scene_of, C * 4});
        parts.push_back({(void**)&s->scene_range, (size_t)s->nscenes * 8});
    }
    size_t total = 0;
    for (auto& pt : parts) total += (pt.second + 255) & ~size_t(255);
    e = lib_malloc(&s->arena, total);
    if (e != cudaSuccess) { delete s; set_error(std::string("cudaMalloc arena: ") + cudaGetErrorString(e)); return PBD_ERR_ALLOC; }
    char* cur = static_cast<char*>(s->arena);
    for (auto& pt : parts) { *pt.first = cur; cur += (pt.second + 255) & ~size_t(255); }
    e = cudaMemset(s->arena, 0, total);
    if (e == cudaSuccess) e = cudaMemset(s->cell_start, 0xFF, T * 4);   // all cells empty
    if (e == cudaSuccess) {                                               // inverse mass 1 everywhere
        for (int b = 0; b < 2; ++b) fill_float_kernel<<<256, 256>>>(s->w[b], 1.0f, capacity);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && s->batched)
        e = cudaMemcpy(s->d_scenes, s->h_scenes.data(), s->nscenes * sizeof(SceneParams), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    auto undo = [&]() {   // a failed create leaves nothing behind
        if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
        cudaFree(s->arena);
        delete s;
    };
    if (e != cudaSuccess) { undo(); return cuda_fail("pbd_create init", e); }
    if (int rc2 = ensure_contacts(s)) { undo(); return rc2; }
    *out = s;
    return PBD_OK;
}
}  // namespace

extern "C" {

int pbd_create(const pbd_params* prm, uint32_t capacity, pbd_sim** out) {
    clear_error();
    if (!prm || !out) { set_error("pbd_create: null argument"); return PBD_ERR_INVALID_ARG; }
    return create_sim(prm, capacity, nullptr, nullptr, out);
}

int pbd_destroy(pbd_sim* s) {
    clear_error();
    if (!s) return PBD_OK;
    cudaDeviceSynchronize();
    destroy_graphs(s);
    for (auto& g : s->adj_graphs) cudaGraphExecDestroy(g.exec);
    if (s->adj_arena) cudaFree(s->adj_arena);
    if (s->ct_arena) cudaFree(s->ct_arena);
    if (s->img_arena) cudaFree(s->img_arena);
    if (s->rb_host) cudaFreeHost(s->rb_host);
    if (s->rb_stream) cudaStreamDestroy(s->rb_stream);
    if (s->rb_fork) cudaEventDestroy(s->rb_fork);
    if (s->rb_join) cudaEventDestroy(s->rb_join);
    if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
    cudaError_t e = cudaFree(s->arena);
    delete s;
    if (e != cudaSuccess) return cuda_fail("cudaFree", e);
    return PBD_OK;
}

int pbd_set_params(pbd_sim* s, const pbd_params* prm) {
    clear_error();
    if (int rc = check_sim(s, "pbd_set_params")) return rc;
    ++s->gen;
    ++s->pgen;
    if (!prm) { set_error("pbd_set_params: null"); return PBD_ERR_INVALID_ARG; }
    if (int rc = pbd_validate_params(prm)) return rc;
    if (prm->max_grid != s->prm.max_grid) { set_error("max_grid is fixed at pbd_create"); return PBD_ERR_UNSUPPORTED; }
    const pbd_params old = s->prm;
    s->prm = *prm;
    if (int rc = ensure_contacts(s)) { s->prm = old; return rc; }
    s->dirty = true;
    return PBD_OK;
}

int pbd_get_params(const pbd_sim* s, pbd_params* prm) {
    if (!s || !prm) { set_error("pbd_get_params: null"); return PBD_ERR_INVALID_ARG; }
    *prm = s->prm;
    return PBD_OK;
}

int pbd_num_particles(const pbd_sim* s, uint32_t* n) {
    if (!s || !n) { set_error("pbd_num_particles: null"); return PBD_ERR_INVALID_ARG; }
    *n = s->N;
    return PBD_OK;
}

int pbd_capacity(const pbd_sim* s, uint32_t* c) {
    if (!s || !c) { set_error("pbd_capacity: null"); return PBD_ERR_INVALID_ARG; }
    *c = s->cap;
    return PBD_OK;
}

static int add_common(pbd_sim* s, uint32_t n, const float* pos4, const float* vel4, const float* col4,
                      const float* inv_mass, cudaMemcpyKind kind, cudaStream_t st, bool sync) {
    ++s->gen;
    s->anchor = -1;
    ++s->pgen;
    if (int rc = check_sim(s, "pbd_add_particles")) return rc;
    if (n == 0) return PBD_OK;
    if (!pos4 || !vel4) { set_error("pbd_add_particles: null position or velocity array"); return PBD_ERR_INVALID_ARG; }
    if (s->batched) { set_error("a batch takes particles per scene: pbd_batch_add_particles"); return PBD_ERR_INVALID_ARG; }
    if ((uint64_t)s->N + n > s->cap) {
        set_error("pbd_add_particles: " + std::to_string(s->N) + " + " + std::to_string(n) + " exceeds capacity " + std::to_string(s->cap));
        return PBD_ERR_CAPACITY;
    }
    const size_t off = s->N, bytes = (size_t)n * 16;
    CK(cudaMemcpyAsync(s->x[s->cur.x] + off, pos4, bytes, kind, st));
    CK(cudaMemcpyAsync(s->v[s->cur.v] + off, vel4, bytes, kind, st));
    if (col4) CK(cudaMemcpyAsync(s->col[s->cur.x] + off, col4, bytes, kind, st));
    if (inv_mass) {
        CK(cudaMemcpyAsync(s->w[s->cur.x] + off, inv_mass, (size_t)n * 4, kind, st));
        if (!s->mass_used) { s->mass_used = true; s->dirty = true; }   // all earlier masses are 1: order-free
    }
    fill_new_kernel<<<div_up(n, 256), 256, 0, st>>>(s->ids[s->cur.x], s->w[s->cur.x], inv_mass != nullptr, s->N, n);
    CK(cudaGetLastError());
    if (sync) CK(cudaStreamSynchronize(st));
    s->N += n;
    s->last_stream = st;
    return PBD_OK;
}

int pbd_add_particles(pbd_sim* s, uint32_t n, const float* pos4, const float* vel4, const float* col4) {
    clear_error();
    if (int rc = check_sim(s, "pbd_add_particles")) return rc;
    // The library's own readback buffers (a host loop feeding pbd_step_readback's output back
    // in): the next write into them is a later frame's readback, queued behind this copy on the
    // same stream (pbd_step and pbd_step_readback first wait for the last stream when they run on
    // another one), so the host need not wait for the copy here.
    const bool own = s->rb_host && pos4 == reinterpret_cast<const float*>(s->rb_host) &&
                     vel4 == reinterpret_cast<const float*>(s->rb_host + s->cap) && !col4;
    return add_common(s, n, pos4, vel4, col4, nullptr, cudaMemcpyHostToDevice, s->last_stream, !own);
}

int pbd_add_particles_mass(pbd_sim* s, uint32_t n, const float* pos4, const float* vel4, const float* col4,
                           const float* inv_mass) {
    clear_error();
    if (int rc = check_sim(s, "pbd_add_particles_mass")) return rc;
    if (!inv_mass) { set_error("pbd_add_particles_mass: null inverse-mass array"); return PBD_ERR_INVALID_ARG; }
    for (uint32_t k = 0; k < n; ++k)
        if (!(inv_mass[k] >= 0.0f) || !std::isfinite(inv_mass[k])) {
            set_error("pbd_add_particles_mass: inverse masses must be finite and >= 0");
            return PBD_ERR_RANGE;
        }
    return add_common(s, n, pos4, vel4, col4, inv_mass, cudaMemcpyHostToDevice, s->last_stream, true);
}

int pbd_add_particles_device(pbd_sim* s, uint32_t n, const float* d_pos4, const float* d_vel4, const float* d_col4, void* stream) {
    clear_error();
    return add_common(s, n, d_pos4, d_vel4, d_col4, nullptr, cudaMemcpyDeviceToDevice, (cudaStream_t)stream, false);
}

int pbd_add_particle(pbd_sim* s, const float pos[3], const float dir[3]) {
    clear_error();
    if (int rc = check_sim(s, "pbd_add_particle")) return rc;
    ++s->gen;
    s->anchor = -1;
    ++s->pgen;
    if (s->batched) { set_error("a batch takes particles per scene: pbd_batch_add_particles"); return PBD_ERR_INVALID_ARG; }
    if (!pos || !dir) { set_error("pbd_add_particle: null"); return PBD_ERR_INVALID_ARG; }
    if ((uint64_t)s->N + 1 > s->cap) { set_error("pbd_add_particle: capacity reached"); return PBD_ERR_CAPACITY; }
    add_one_kernel<<<1, 1, 0, s->last_stream>>>(s->x[s->cur.x], s->v[s->cur.v], s->col[s->cur.x], s->ids[s->cur.x],
                                                 s->w[s->cur.x], s->N,
                                                 pos[0], pos[1], pos[2], dir[0], dir[1], dir[2]);
    CK(cudaGetLastError());
    s->N += 1;
    return PBD_OK;
}

int pbd_clear(pbd_sim* s) {
    clear_error();
    if (int rc = check_sim(s, "pbd_clear")) return rc;
    ++s->gen;
    s->anchor = -1;
    ++s->pgen;
    s->N = 0;   // Communication.h:657-660
    std::fill(s->scene_count.begin(), s->scene_count.end(), 0u);
    return PBD_OK;
}

int pbd_step(pbd_sim* s, int nsteps, void* stream) {
    clear_error();
    if (int rc = check_sim(s, "pbd_step")) return rc;
    ++s->gen;
    if (nsteps < 0) { set_error("pbd_step: nsteps < 0"); return PBD_ERR_INVALID_ARG; }
    if (s->N == 0 || nsteps == 0) return PBD_OK;   // Fluid.cu:19
    cudaStream_t st = (cudaStream_t)stream;
    if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));   // work queued on another stream
    if (s->dirty || s->graph_n != s->N || s->table_passes != sort_passes(s)) {
        if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));
        if (int rc = settle_tables(s, st)) return rc;
        if (int rc = build_graphs(s)) return rc;
    }
    for (int k = 0; k < nsteps; ++k) {
        int g = -1;
        for (int j = 0; j < s->nexec; ++j)
            if (s->exec_start[j] == s->cur) { g = j; break; }
        if (g < 0) {   // state moved outside the recorded cycle (a debug front): record again
            if (int rc = build_graphs(s)) return rc;
            g = 0;
        }
        s->anchor = (s->cur.p + 1) % 3;   // this frame's anchor buffer (see enqueue_frame)
        CK(cudaGraphLaunch(s->exec[g], st));
        s->cur = s->exec_end[g];
    }
    s->table_hint = s->N;
    s->last_stream = st;
    return PBD_OK;
}

int pbd_step_readback(pbd_sim* s, int nsteps, void* stream, const float** pos4, const float** vel4) {
    clear_error();
    if (int rc = check_sim(s, "pbd_step_readback")) return rc;
    if (nsteps < 1) { set_error("pbd_step_readback: nsteps < 1"); return PBD_ERR_INVALID_ARG; }
    if (s->batched) { set_error("pbd_step_readback: a batch reads its scenes with pbd_batch_get_state"); return PBD_ERR_INVALID_ARG; }
    if (!s->rb_host) {
        if (cudaError_t ea = lib_host_alloc((void**)&s->rb_host, (size_t)2 * s->cap * 16, cudaHostAllocMapped)) {
            s->rb_host = nullptr;
            set_error(std::string("pbd_step_readback: pinned host buffers: ") + cudaGetErrorString(ea));
            return PBD_ERR_ALLOC;
        }
        CK(cudaHostGetDevicePointer((void**)&s->rb_dev, s->rb_host, 0));
        CK(cudaStreamCreateWithFlags(&s->rb_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&s->rb_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&s->rb_join, cudaEventDisableTiming));
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (s->N > 0) {
        if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));   // work queued on another stream
        if (nsteps > 1)
            if (int rc = pbd_step(s, nsteps - 1, stream)) return rc;
        ++s->gen;
        if (s->dirty || s->graph_n != s->N || s->table_passes != sort_passes(s)) {
            if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));
            if (int rc = settle_tables(s, st)) return rc;
            if (int rc = build_graphs(s)) return rc;
        }
        int g = -1;
        for (int j = 0; j < s->nexec; ++j)
            if (s->exec_start[j] == s->cur) { g = j; break; }
        if (g < 0) {
            if (int rc = build_graphs(s)) return rc;
            g = 0;
        }
        if (s->rb_n != s->nexec)
            if (int rc = build_rb_graphs(s)) return rc;
        s->anchor = (s->cur.p + 1) % 3;
        CK(cudaGraphLaunch(s->rb_exec[g], st));
        s->cur = s->exec_end[g];
        s->table_hint = s->N;
        s->last_stream = st;
        CK(cudaStreamSynchronize(st));
    }
    if (pos4) *pos4 = reinterpret_cast<const float*>(s->rb_host);
    if (vel4) *vel4 = reinterpret_cast<const float*>(s->rb_host + s->cap);
    return PBD_OK;
}

int pbd_sync(pbd_sim* s) {
    clear_error();
    if (int rc = check_sim(s, "pbd_sync")) return rc;
    if (int rc = sync_last(s)) return rc;
    uint32_t err = 0;
    CK(cudaMemcpy(&err, s->err, 4, cudaMemcpyDeviceToHost));
    if (err) {
        CK(cudaMemset(s->err, 0, 4));
        if (err & kErrSortTimeout) { set_error("radix sort: a bounded look-back wait gave up"); return PBD_ERR_TIMEOUT; }
        set_error("Morton keys exceed the sorted bit range");
        return PBD_ERR_RANGE;
    }
    return PBD_OK;
}

int pbd_get_state(pbd_sim* s, float* pos4, float* vel4, float* pred4, uint32_t* ids) {
    clear_error();
    if (int rc = check_sim(s, "pbd_get_state")) return rc;
    if (int rc = sync_last(s)) return rc;
    const size_t b = (size_t)s->N * 16;
    if (pos4) CK(cudaMemcpy(pos4, s->x[s->cur.x], b, cudaMemcpyDeviceToHost));
    if (vel4) CK(cudaMemcpy(vel4, s->v[s->cur.v], b, cudaMemcpyDeviceToHost));
    if (pred4) CK(cudaMemcpy(pred4, s->p[s->cur.p], b, cudaMemcpyDeviceToHost));
    if (ids) CK(cudaMemcpy(ids, s->ids[s->cur.x], (size_t)s->N * 4, cudaMemcpyDeviceToHost));
    return PBD_OK;
}

int pbd_get_device_state(pbd_sim* s, const float** d_pos4, const float** d_vel4, const float** d_pred4) {
    clear_error();
    if (int rc = check_sim(s, "pbd_get_device_state")) return rc;
    if (d_pos4) *d_pos4 = reinterpret_cast<const float*>(s->x[s->cur.x]);
    if (d_vel4) *d_vel4 = reinterpret_cast<const float*>(s->v[s->cur.v]);
    if (d_pred4) *d_pred4 = reinterpret_cast<const float*>(s->p[s->cur.p]);
    return PBD_OK;
}

int pbd_debug_dump(pbd_sim* s, uint32_t* keys, uint32_t* perm, uint32_t* cell_start, uint32_t* cell_end,
                   uint32_t ncells, float* lambda, float* fext4, float* omega4) {
    clear_error();
    if (int rc = check_sim(s, "pbd_debug_dump")) return rc;
    if (int rc = sync_last(s)) return rc;
    const int fin = (s->table_passes >= 0 ? s->table_passes : sort_passes(s)) % 2;
    const size_t n = s->N;
    if (keys) CK(cudaMemcpy(keys, s->keys[fin], n * 4, cudaMemcpyDeviceToHost));
    if (perm) CK(cudaMemcpy(perm, s->vals[fin], n * 4, cudaMemcpyDeviceToHost));
    if (ncells > s->prm.max_grid) ncells = s->prm.max_grid;
    if (cell_start) CK(cudaMemcpy(cell_start, s->cell_start, (size_t)ncells * 4, cudaMemcpyDeviceToHost));
    if (cell_end) CK(cudaMemcpy(cell_end, s->cell_end, (size_t)ncells * 4, cudaMemcpyDeviceToHost));
    if (lambda) CK(cudaMemcpy(lambda, s->lambda, n * 4, cudaMemcpyDeviceToHost));
    if (fext4) CK(cudaMemcpy(fext4, s->fext, n * 16, cudaMemcpyDeviceToHost));
    if (omega4) CK(cudaMemcpy(omega4, s->omega, n * 16, cudaMemcpyDeviceToHost));
    return PBD_OK;
}

int pbd_debug_neighbours(pbd_sim* s, uint32_t max_entries, uint32_t* list, uint32_t* count, uint32_t* contacts,
                         int walker) {
    clear_error();
    if (int rc = check_sim(s, "pbd_debug_neighbours")) return rc;
    if (int rc = sync_last(s)) return rc;
    const size_t n = s->N;
    if (n == 0) return PBD_OK;
    uint32_t *dl = nullptr, *dc = nullptr, *dk = nullptr;
    const size_t lb = std::max<size_t>(1, n * (size_t)max_entries) * 4;
    cudaError_t ea = lib_malloc((void**)&dl, lb);
    if (ea == cudaSuccess) ea = lib_malloc((void**)&dc, n * 4);
    if (ea == cudaSuccess) ea = lib_malloc((void**)&dk, n * 4);
    if (ea != cudaSuccess) {
        if (dl) cudaFree(dl);
        if (dc) cudaFree(dc);
        set_error(std::string("pbd_debug_neighbours: ") + cudaGetErrorString(ea));
        return PBD_ERR_ALLOC;
    }
    CK(cudaMemsetAsync(dl, 0, lb, s->last_stream));   // slots past each count read back as 0
    const DevParams P = make_dev_params(s);
    const bool cols = (s->prm.flags & PBD_FLAG_COLORS) && (s->prm.active & PBD_ACTIVE_FIND_NEIGHBOURS);
    const uint32_t threads = walker ? (uint32_t)n * 32u : (uint32_t)n;
    list_kernel<<<div_up(threads, 128), 128, 0, s->last_stream>>>(P, s->p[s->cur.p], s->cell_start, s->cell_end,
                                                                  max_entries, dl, dc, dk,
                                                                  cols ? s->col[s->cur.x] : nullptr, walker ? 1 : 0);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->last_stream);
    if (e == cudaSuccess && list) e = cudaMemcpy(list, dl, n * (size_t)max_entries * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && count) e = cudaMemcpy(count, dc, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && contacts) e = cudaMemcpy(contacts, dk, n * 4, cudaMemcpyDeviceToHost);
    cudaFree(dl); cudaFree(dc); cudaFree(dk);
    if (e != cudaSuccess) return cuda_fail("pbd_debug_neighbours", e);
    return PBD_OK;
}

int pbd_debug_fail_allocations(uint32_t skip, uint32_t fail) {
    std::lock_guard<std::mutex> lock(pbd::g_alloc_mutex);
    pbd::g_alloc_skip = fail ? skip : 0u;
    pbd::g_alloc_fail = fail;
    return PBD_OK;
}

int pbd_debug_set_wait_limit(pbd_sim* s, uint32_t spins, int hold_first_tile) {
    clear_error();
    if (!s) return pbd_noalloc_set_wait_limit(spins, hold_first_tile);
    if (int rc = check_sim(s, "pbd_debug_set_wait_limit")) return rc;
    s->sort_spin_limit = spins ? spins : kSpinLimit;
    s->sort_hold = hold_first_tile ? 1u : 0u;
    s->dirty = true;   // the frame graphs hold the sort's settings
    return PBD_OK;
}

int pbd_debug_front(pbd_sim* s, void* stream) {
    clear_error();
    if (int rc = check_sim(s, "pbd_debug_front")) return rc;
    ++s->gen;
    if (s->N == 0) return PBD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));
    if (int rc = settle_tables(s, st)) return rc;
    uint32_t nl = 0;
    s->anchor = (s->cur.p + 1) % 3;
    cudaError_t e = enqueue_frame(s, st, s->cur, true, nl);
    if (e != cudaSuccess) return cuda_fail("pbd_debug_front", e);
    CK(cudaStreamSynchronize(st));
    s->table_hint = s->N;
    s->last_stream = st;
    return PBD_OK;
}

int pbd_profile_frames(pbd_sim* s, int nsteps, void* stream, pbd_kernel_stat* stats, uint32_t max_stats,
                       uint32_t* n_stats) {
    clear_error();
    if (int rc = check_sim(s, "pbd_profile_frames")) return rc;
    ++s->gen;
    if (!stats || !n_stats || nsteps < 0) { set_error("pbd_profile_frames: bad argument"); return PBD_ERR_INVALID_ARG; }
    *n_stats = 0;
    if (s->N == 0 || nsteps == 0) return PBD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));
    if (int rc = settle_tables(s, st)) return rc;
    Profiler prof;
    prof.st = st;
    for (int k = 0; k < nsteps; ++k) {
        uint32_t nl = 0;
        s->anchor = (s->cur.p + 1) % 3;
        cudaError_t e = enqueue_frame(s, st, s->cur, false, nl, &prof);
        if (e != cudaSuccess) return cuda_fail("pbd_profile_frames", e);
        s->table_hint = s->N;
    }
    s->last_stream = st;
    CK(cudaStreamSynchronize(st));
    uint32_t n = 0;
    for (auto& r : prof.recs) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, r.a, r.b));
        uint32_t k = 0;
        while (k < n && std::strncmp(stats[k].name, r.name, sizeof(stats[k].name)) != 0) ++k;
        if (k == n) {
            if (n == max_stats) continue;
            std::memset(&stats[n], 0, sizeof(stats[n]));
            std::strncpy(stats[n].name, r.name, sizeof(stats[n].name) - 1);
            ++n;
        }
        stats[k].launches += 1;
        stats[k].total_ms += ms;
    }
    *n_stats = n;
    return PBD_OK;
}

static int density_error_impl(pbd_sim* s, const char* who, float* err, uint32_t min_nb, float margin, double* out,
                              void* stream) {
    clear_error();
    if (int rc = check_sim(s, who)) return rc;
    for (int k = 0; k < 5; ++k) out[k] = 0.0;
    if (s->N == 0) return PBD_OK;
    if (s->anchor < 0) {
        set_error(std::string(who) + ": run a frame (pbd_step) after the last change of the state");
        return PBD_ERR_INVALID_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));
    const DevParams P = make_dev_params(s);
    const uint32_t N = s->N;
    CK(cudaMemsetAsync(s->stats, 0, 40, st));
    density_error_kernel<<<div_up(N, 128), 128, 0, st>>>(P, s->p[s->cur.p], s->p[s->anchor], s->cell_start, s->cell_end,
                                                          s->lambda, s->stats, min_nb, margin);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, s->stats, 40, cudaMemcpyDeviceToHost, st));
    if (err) CK(cudaMemcpyAsync(err, s->lambda, (size_t)N * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    s->last_stream = st;
    return PBD_OK;
}

int pbd_density_error(pbd_sim* s, float* err, double* mean_abs, double* max_abs, void* stream) {
    double acc[5];
    if (int rc = density_error_impl(s, "pbd_density_error", err, 0xFFFFFFFFu, 0.0f, acc, stream)) return rc;
    if (mean_abs) *mean_abs = s->N ? acc[0] / (double)s->N : 0.0;
    if (max_abs) *max_abs = acc[1];
    return PBD_OK;
}

int pbd_density_error_interior(pbd_sim* s, uint32_t min_neighbours, float margin, double* mean_abs, double* max_abs,
                               uint32_t* counted, void* stream) {
    if (!(margin >= 0.0f)) { set_error("pbd_density_error_interior: margin must be >= 0"); return PBD_ERR_INVALID_ARG; }
    double acc[5];
    if (int rc = density_error_impl(s, "pbd_density_error_interior", nullptr, min_neighbours, margin, acc, stream)) return rc;
    const double n = acc[4];
    if (mean_abs) *mean_abs = n > 0.0 ? acc[2] / n : 0.0;
    if (max_abs) *max_abs = acc[3];
    if (counted) *counted = (uint32_t)n;
    return PBD_OK;
}

int pbd_render_sprites(pbd_sim* s, const pbd_camera* cam, uint8_t* rgba, float* depth, void* stream) {
    clear_error();
    if (int rc = check_sim(s, "pbd_render_sprites")) return rc;
    if (!cam || cam->width == 0 || cam->height == 0 || (size_t)cam->width * cam->height > (size_t(1) << 28)) {
        set_error("pbd_render_sprites: camera size must be in [1, 2^28] pixels");
        return PBD_ERR_INVALID_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));
    const size_t npx = (size_t)cam->width * cam->height;
    const size_t need = npx * 8 + ((npx * 4 + 255) & ~size_t(255)) * 2 + 256;
    if (need > s->img_bytes) {
        CK(cudaStreamSynchronize(st));
        if (s->img_arena) cudaFree(s->img_arena);
        s->img_arena = nullptr;
        cudaError_t e = lib_malloc(&s->img_arena, need);
        if (e != cudaSuccess) { s->img_bytes = 0; set_error(std::string("sprite image: ") + cudaGetErrorString(e)); return PBD_ERR_ALLOC; }
        s->img_bytes = need;
    }
    unsigned long long* key = static_cast<unsigned long long*>(s->img_arena);
    uint32_t* d_rgba = reinterpret_cast<uint32_t*>(static_cast<char*>(s->img_arena) + npx * 8);
    float* d_depth = reinterpret_cast<float*>(reinterpret_cast<char*>(d_rgba) + ((npx * 4 + 255) & ~size_t(255)));
    SpriteCam c{};
    std::memcpy(c.V, cam->view, sizeof(c.V));
    std::memcpy(c.Pm, cam->projection, sizeof(c.Pm));
    for (int k = 0; k < 3; ++k) { c.vd[k] = -cam->view_direction[k]; c.light[k] = cam->light_position[k]; }
    c.r = cam->sphere_radius;
    c.W = cam->width;
    c.H = cam->height;
    const uint32_t gs = std::max(1u, std::min((uint32_t)div_up(npx, 256), (uint32_t)s->num_sms * 16u));
    sprite_clear_kernel<<<gs, 256, 0, st>>>(key, npx, make_float4(cam->clear_rgba[0], cam->clear_rgba[1],
                                                                    cam->clear_rgba[2], cam->clear_rgba[3]));
    if (s->N) sprite_splat_kernel<<<div_up(s->N, 256), 256, 0, st>>>(c, s->x[s->cur.x], s->col[s->cur.x], s->N, key);
    sprite_resolve_kernel<<<(uint32_t)div_up(npx, 256), 256, 0, st>>>(key, cam->width, cam->height, d_rgba, d_depth);
    CK(cudaGetLastError());
    if (rgba) CK(cudaMemcpyAsync(rgba, d_rgba, npx * 4, cudaMemcpyDeviceToHost, st));
    if (depth) CK(cudaMemcpyAsync(depth, d_depth, npx * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    s->last_stream = st;
    return PBD_OK;
}

int pbd_launches_per_step(pbd_sim* s, uint32_t* n) {
    clear_error();
    if (int rc = check_sim(s, "pbd_launches_per_step")) return rc;
    if (!n) { set_error("pbd_launches_per_step: null"); return PBD_ERR_INVALID_ARG; }
    if (s->dirty || s->graph_n != s->N) {
        if (s->N == 0) { *n = 0; return PBD_OK; }
        if (int rc = build_graphs(s)) return rc;
    }
    *n = s->launches;
    return PBD_OK;
}


// ======================================================================================
// Block-size tuning of the neighbour passes, with a JSON-lines cache
// ======================================================================================
namespace {
std::string tune_signature(const pbd_sim* s) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "n=%u;scenes=%u;iters=%u;stab=%u;active=%u;M=%u;K=%u;hs=%g;hp=%g;d=%g;mass=%d",
                  s->N, s->nscenes, s->prm.solver_iterations, s->prm.stabilization_iterations, s->prm.active,
                  s->prm.max_neighbours_per_particle, s->prm.kernel_width_neighbours, s->prm.kernel_width_spiky,
                  s->prm.kernel_width_poly, 2.0 * s->prm.particle_radius, s->mass_used ? 1 : 0);
    return buf;
}

bool cache_lookup(const char* path, const std::string& sig, int* block) {
    if (!path) return false;
    FILE* f = std::fopen(path, "r");
    if (!f) return false;
    char line[1024];
    bool found = false;
    const std::string key = "\"signature\": \"" + sig + "\"";
    while (std::fgets(line, sizeof(line), f)) {
        if (std::strstr(line, key.c_str())) {
            const char* b = std::strstr(line, "\"block\": ");
            if (b) { *block = std::atoi(b + 9); found = true; }
        }
    }
    std::fclose(f);
    return found && (*block == 64 || *block == 128 || *block == 256);
}
}  // namespace

int pbd_autotune(pbd_sim* s, const char* cache_path, void* stream, uint32_t* block) {
    clear_error();
    if (int rc = check_sim(s, "pbd_autotune")) return rc;
    ++s->gen;
    s->anchor = -1;
    ++s->pgen;
    if (s->N == 0) { set_error("pbd_autotune: no particles"); return PBD_ERR_INVALID_ARG; }
    const std::string sig = tune_signature(s);
    int best = 0;
    if (!cache_lookup(cache_path, sig, &best)) {
        cudaStream_t st = (cudaStream_t)stream;
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        float best_ms = 1e30f;
        for (int tpb : {64, 128, 256}) {
            s->tpb_nbr = tpb;
            s->dirty = true;
            if (int rc = pbd_step(s, 2, stream)) return rc;        // records the graphs, warms up
            CK(cudaEventRecord(a, st));
            if (int rc = pbd_step(s, 3, stream)) return rc;
            CK(cudaEventRecord(b, st));
            CK(cudaEventSynchronize(b));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, a, b));
            if (ms < best_ms) { best_ms = ms; best = tpb; }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if (cache_path) {
            FILE* f = std::fopen(cache_path, "a");
            if (f) {
                std::fprintf(f, "{\"signature\": \"%s\", \"block\": %d, \"frame_ms\": %.6f}\n", sig.c_str(), best, best_ms / 3.0f);
                std::fclose(f);
            }
        }
    }
    s->tpb_nbr = best;
    s->dirty = true;
    if (block) *block = (uint32_t)best;
    return PBD_OK;
}

// ======================================================================================
// Batched scenes: one simulation whose particles carry a scene number
// ======================================================================================
static pbd_sim* as_sim(pbd_batch* b) { return reinterpret_cast<pbd_sim*>(b); }

int pbd_batch_create(const pbd_params* shared, uint32_t nscenes, const pbd_scene_desc* scenes, pbd_batch** out) {
    clear_error();
    if (!shared || !scenes || !out || nscenes == 0) { set_error("pbd_batch_create: bad argument"); return PBD_ERR_INVALID_ARG; }
    *out = nullptr;
    if (shared->max_grid != 128u * 128u * 128u) { set_error("pbd_batch_create: scenes use the 128^3 grid (max_grid)"); return PBD_ERR_UNSUPPORTED; }
    std::vector<SceneParams> sp(nscenes);
    std::vector<uint32_t> caps(nscenes);
    uint64_t total = 0, cells = 0;
    for (uint32_t k = 0; k < nscenes; ++k) {
        pbd_params q = *shared;   // each scene's values are checked with the reference's ranges
        q.rest_density = scenes[k].rest_density;
        q.gravity = scenes[k].gravity;
        for (int a = 0; a < 3; ++a) { q.bounds_min[a] = scenes[k].bounds_min[a]; q.bounds_max[a] = scenes[k].bounds_max[a]; }
        if (int rc = pbd_validate_params(&q)) {
            set_error("scene " + std::to_string(k) + ": " + pbd_last_error());
            return rc;
        }
        sp[k].rho0 = scenes[k].rest_density;
        sp[k].gravity = scenes[k].gravity;
        for (int a = 0; a < 3; ++a) { sp[k].bmin[a] = scenes[k].bounds_min[a]; sp[k].bmax[a] = scenes[k].bounds_max[a]; }
        // the scene's slice of the cell tables: every Morton key of a cell its walls enclose (keys
        // come from positions clamped to the walls; the key grows with each coordinate, so the
        // far corner's key is the largest)
        const uint32_t tx = (uint32_t)std::min(127.f, std::max(0.f, scenes[k].bounds_max[0]));
        const uint32_t ty = (uint32_t)std::min(127.f, std::max(0.f, scenes[k].bounds_max[1]));
        const uint32_t tz = (uint32_t)std::min(127.f, std::max(0.f, scenes[k].bounds_max[2]));
        sp[k].base = (uint32_t)cells;
        sp[k].cells = (host_expand_bits(tx) << 2) + (host_expand_bits(ty) << 1) + host_expand_bits(tz) + 1u;
        cells += sp[k].cells;
        if (cells > (1ull << 32) - 1) { set_error("pbd_batch_create: the scenes' cell tables exceed 2^32 cells"); return PBD_ERR_RANGE; }
        caps[k] = scenes[k].capacity;
        total += scenes[k].capacity;
    }
    if (total == 0 || total > (1u << 30) - 1u) { set_error("pbd_batch_create: total capacity must be in [1, 2^30)"); return PBD_ERR_INVALID_ARG; }
    pbd_sim* s = nullptr;
    int rc = create_sim(shared, (uint32_t)total, &sp, &caps, &s);
    if (rc) return rc;
    *out = reinterpret_cast<pbd_batch*>(s);
    return PBD_OK;
}

int pbd_batch_destroy(pbd_batch* b) { return pbd_destroy(as_sim(b)); }

int pbd_batch_add_particles(pbd_batch* b, uint32_t scene, uint32_t n, const float* pos4, const float* vel4) {
    clear_error();
    pbd_sim* s = as_sim(b);
    if (int rc = check_sim(s, "pbd_batch_add_particles")) return rc;
    if (scene >= s->nscenes) { set_error("pbd_batch_add_particles: scene out of range"); return PBD_ERR_INVALID_ARG; }
    if (n == 0) return PBD_OK;
    if (!pos4 || !vel4) { set_error("pbd_batch_add_particles: null array"); return PBD_ERR_INVALID_ARG; }
    if ((uint64_t)s->scene_count[scene] + n > s->scene_cap[scene]) {
        set_error("pbd_batch_add_particles: scene " + std::to_string(scene) + " capacity " + std::to_string(s->scene_cap[scene]) + " exceeded");
        return PBD_ERR_CAPACITY;
    }
    cudaStream_t st = s->last_stream;
    const size_t off = s->N, bytes = (size_t)n * 16;
    CK(cudaMemcpyAsync(s->x[s->cur.x] + off, pos4, bytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->v[s->cur.v] + off, vel4, bytes, cudaMemcpyHostToDevice, st));
    fill_new_kernel<<<div_up(n, 256), 256, 0, st>>>(s->ids[s->cur.x], s->w[s->cur.x], 0, s->N, n);
    fill_u32_kernel<<<div_up(n, 256), 256, 0, st>>>(s->scene_of, scene, s->N, n);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    s->N += n;
    s->scene_count[scene] += n;
    return PBD_OK;
}

int pbd_batch_step(pbd_batch* b, int nsteps, void* stream) { return pbd_step(as_sim(b), nsteps, stream); }
int pbd_batch_sync(pbd_batch* b) { return pbd_sync(as_sim(b)); }
int pbd_batch_num_particles(pbd_batch* b, uint32_t scene, uint32_t* n) {
    clear_error();
    pbd_sim* s = as_sim(b);
    if (int rc = check_sim(s, "pbd_batch_num_particles")) return rc;
    if (!n || scene >= s->nscenes) { set_error("pbd_batch_num_particles: bad argument"); return PBD_ERR_INVALID_ARG; }
    *n = s->scene_count[scene];
    return PBD_OK;
}

int pbd_batch_get_state(pbd_batch* b, uint32_t scene, float* pos4, float* vel4) {
    clear_error();
    pbd_sim* s = as_sim(b);
    if (int rc = check_sim(s, "pbd_batch_get_state")) return rc;
    if (scene >= s->nscenes) { set_error("pbd_batch_get_state: scene out of range"); return PBD_ERR_INVALID_ARG; }
    if (int rc = sync_last(s)) return rc;
    const size_t N = s->N;
    std::vector<float4> x(N), v(N);
    std::vector<uint32_t> sc(N);
    CK(cudaMemcpy(x.data(), s->x[s->cur.x], N * 16, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(v.data(), s->v[s->cur.v], N * 16, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(sc.data(), s->scene_of, N * 4, cudaMemcpyDeviceToHost));
    size_t k = 0;
    for (size_t i = 0; i < N; ++i) {
        if (sc[i] != scene) continue;
        if (pos4) std::memcpy(pos4 + 4 * k, &x[i], 16);
        if (vel4) std::memcpy(vel4 + 4 * k, &v[i], 16);
        ++k;
    }
    return PBD_OK;
}

int pbd_batch_autotune(pbd_batch* b, const char* cache_path, void* stream, uint32_t* block) {
    return pbd_autotune(as_sim(b), cache_path, stream, block);
}

int pbd_batch_launches_per_step(pbd_batch* b, uint32_t* n) { return pbd_launches_per_step(as_sim(b), n); }

int pbd_batch_profile_frames(pbd_batch* b, int nsteps, void* stream, pbd_kernel_stat* stats, uint32_t max_stats,
                             uint32_t* n_stats) {
    return pbd_profile_frames(as_sim(b), nsteps, stream, stats, max_stats, n_stats);
}


// ======================================================================================
// Adjoint (no counterpart in the reference): checkpointed forward, taped recompute, reverse
// ======================================================================================
static int adjoint_supported(const pbd_sim* s) {
    const pbd_params& p = s->prm;
    const uint32_t need = PBD_ACTIVE_APPLY_FORCES | PBD_ACTIVE_FIND_CONTACTS | PBD_ACTIVE_COMPUTE_LAMBDA |
                          PBD_ACTIVE_COMPUTE_DELTA_POSITIONS | PBD_ACTIVE_APPLY_DELTA_POSITIONS | PBD_ACTIVE_UPDATE_POSITIONS;
    if ((p.active & need) != need) { set_error("adjoint: applyForces, findContacts, computeLambda, computeDeltaPositions, applyDeltaPositions and updatePositions must be active"); return PBD_ERR_UNSUPPORTED; }
    if ((p.active & PBD_ACTIVE_COMPUTE_VORTICITY) && !(p.active & PBD_ACTIVE_COMPUTE_OMEGAS)) {
        set_error("adjoint: vorticity needs computeOmegas (it would read a stale omega)");
        return PBD_ERR_UNSUPPORTED;
    }
    if (p.stabilization_iterations > (uint32_t)kMaxTapeStab || p.solver_iterations == 0 ||
        p.solver_iterations > (uint32_t)kMaxTapeIters) {
        set_error("adjoint: stabilizationIterations must be 0..8 and solverIterations 1..16");
        return PBD_ERR_UNSUPPORTED;
    }
    if (s->batched) { set_error("adjoint: batches have no reverse pass"); return PBD_ERR_UNSUPPORTED; }
    if (p.collision_type != 0) { set_error("adjoint: collisionType 1 has no reverse pass"); return PBD_ERR_UNSUPPORTED; }
    return PBD_OK;
}

static int adj_segment(pbd_sim* s, cudaStream_t st, int nf, int kind);

int pbd_adjoint_forward(pbd_sim* s, int nsteps, int ckpt_every, void* stream) {
    clear_error();
    if (int rc = check_sim(s, "pbd_adjoint_forward")) return rc;
    if (nsteps < 1 || ckpt_every < 1) { set_error("pbd_adjoint_forward: nsteps and ckpt_every must be >= 1"); return PBD_ERR_INVALID_ARG; }
    if (s->N == 0) { set_error("pbd_adjoint_forward: no particles"); return PBD_ERR_INVALID_ARG; }
    if (int rc = adjoint_supported(s)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));
    const size_t N = s->N;
    const int k = std::min(ckpt_every, nsteps);
    const int nck = (nsteps + k - 1) / k;
    const uint32_t I = s->prm.solver_iterations;
    // workspace: checkpoints, the final state, k frames of tape, gradient buffers
    const bool visc = (s->prm.active & PBD_ACTIVE_COMPUTE_VISCOSITY) != 0;
    const bool solids = s->mass_used != 0;
    const bool vort = (s->prm.active & PBD_ACTIVE_COMPUTE_VORTICITY) != 0;
    const bool tape_full = visc || vort;   // the reverse passes after updatePositions read the frame's full list
    const uint32_t S = s->prm.stabilization_iterations;
    const bool stab_tape = s->prm.collision_type == 0 && S > 1;   // contact passes after the first
    const size_t per_tape = N * (16 + 16 + 4 + 4 + ((visc || vort) ? 32 : 0) + (solids ? 4 : 0) + (vort ? 48 : 0)) +
                            (tape_full ? N * (4 * (size_t)s->fl_slots + 4) : 0) +
                            (size_t)I * N * (16 + 4 + 32 + 4 * kListMax + 4) +
                            (stab_tape ? (size_t)I * (S - 1) * (N * 16 + 256) : 0) + 2048;
    const size_t acc_bytes = 16 * (size_t)div_up((uint32_t)N, 128);   // two doubles per reverse block
    const size_t w_bytes = solids ? ((size_t)nck + 1) * N * 4 + 512 : 0;   // checkpoints + final
    const size_t vort_bytes = (vort ? N * 48 + ((size_t)nck + 1) * N * 16 + 1024 : 0) +
                              (stab_tape ? N * 32 + 256 : 0);   // scat3, gom, force checkpoints
    const size_t need = (size_t)nck * N * 32 + N * 64 + N * 8 + (size_t)k * per_tape + 6 * N * 16 + N * 4 + acc_bytes + w_bytes + vort_bytes +
                        N * 64 + (size_t)(19 + (4 + 5 * I) * k) * 256;
    if (need > s->adj_bytes) {
        if (s->adj_arena) CK(cudaStreamSynchronize(st));
        if (s->adj_arena) cudaFree(s->adj_arena);
        s->adj_arena = nullptr;
        cudaError_t e = lib_malloc(&s->adj_arena, need);
        if (e != cudaSuccess) { s->adj_bytes = 0; set_error(std::string("adjoint workspace: ") + cudaGetErrorString(e)); return PBD_ERR_ALLOC; }
        s->adj_bytes = need;
    }
    char* c = static_cast<char*>(s->adj_arena);
    auto take = [&](size_t bytes) { char* r = c; c += (bytes + 255) & ~size_t(255); return r; };
    s->adj_ck_x = (float4*)take((size_t)nck * N * 16);
    s->adj_ck_v = (float4*)take((size_t)nck * N * 16);
    s->adj_fin_x = (float4*)take(N * 16);
    s->adj_fin_v = (float4*)take(N * 16);
    s->adj_fin_p = (float4*)take(N * 16);
    s->adj_fin_col = (float4*)take(N * 16);
    s->adj_fin_keys = (uint32_t*)take(N * 4);
    s->adj_fin_ids = (uint32_t*)take(N * 4);
    s->adj_ck_w = solids ? (float*)take((size_t)nck * N * 4) : nullptr;
    s->adj_fin_w = solids ? (float*)take(N * 4) : nullptr;
    s->adj_ck_f = vort ? (float4*)take((size_t)nck * N * 16) : nullptr;
    s->adj_fin_f = vort ? (float4*)take(N * 16) : nullptr;
    s->adj_tape.assign(k, Tape{});
    for (int t = 0; t < k; ++t) {
        Tape& T = s->adj_tape[t];
        T.x_in = (float4*)take(N * 16);
        T.v_in = (float4*)take(N * 16);
        T.perm = (uint32_t*)take(N * 4);
        T.keys = (uint32_t*)take(N * 4);
        for (uint32_t it = 0; it < I; ++it) {
            for (uint32_t k = 0; k + 1 < (uint32_t)kMaxTapeStab; ++k)
                T.p_s[it][k] = (stab_tape && k + 1 < S) ? (float4*)take(N * 16) : nullptr;
            T.p_it[it] = (float4*)take(N * 16);
            T.lam[it] = (float*)take(N * 4);
            T.aux[it] = (float4*)take(N * 32);
            T.near[it] = (uint32_t*)take(N * 4 * kListMax);
            T.near_meta[it] = (uint32_t*)take(N * 4);
        }
        T.p_fin = (visc || vort) ? (float4*)take(N * 16) : nullptr;
        T.v_u = (visc || vort) ? (float4*)take(N * 16) : nullptr;
        T.w = solids ? (float*)take(N * 4) : nullptr;
        T.omega = vort ? (float4*)take(N * 16) : nullptr;
        T.eta = vort ? (float4*)take(N * 16) : nullptr;
        T.full = tape_full ? (uint32_t*)take(N * 4 * (size_t)s->fl_slots) : nullptr;
        T.full_meta = tape_full ? (uint32_t*)take(N * 4) : nullptr;
        T.fext = vort ? (float4*)take(N * 16) : nullptr;
    }
    for (int g = 0; g < 6; ++g) s->adj_g[g] = (float4*)take(N * 16);
    s->adj_glam = (float*)take(N * 4);
    s->adj_acc = (double*)take(acc_bytes);
    s->adj_gmax = (uint32_t*)take(4);
    s->adj_scat = (unsigned long long*)take((size_t)N * 32);
    s->adj_scat2 = (unsigned long long*)take((size_t)N * 32);
    s->adj_scat3 = (vort || stab_tape) ? (unsigned long long*)take((size_t)N * 32) : nullptr;
    s->adj_gom = vort ? (float4*)take((size_t)N * 16) : nullptr;
    s->adj_steps = nsteps;
    s->adj_every = k;
    s->adj_nck = nck;
    s->adj_n = s->N;
    s->adj_last_taped = false;
    for (int ck = 0; ck < nck; ++ck) {
        const int nf = std::min(k, nsteps - ck * k);
        CK(cudaMemcpyAsync(s->adj_ck_x + (size_t)ck * N, s->x[s->cur.x], N * 16, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(s->adj_ck_v + (size_t)ck * N, s->v[s->cur.v], N * 16, cudaMemcpyDeviceToDevice, st));
        if (solids)   // the re-order permutes the inverse masses with the state
            CK(cudaMemcpyAsync(s->adj_ck_w + (size_t)ck * N, s->w[s->cur.x], N * 4, cudaMemcpyDeviceToDevice, st));
        if (vort)     // the vorticity force the segment's first frame applies
            CK(cudaMemcpyAsync(s->adj_ck_f + (size_t)ck * N, s->fext, N * 16, cudaMemcpyDeviceToDevice, st));
        if (ck + 1 < nck) {
            if (int rc = pbd_step(s, nf, stream)) return rc;
        } else {
            // the last segment keeps its tape now, so the reverse pass need not recompute it
            if (s->dirty || s->graph_n != s->N || s->table_passes != sort_passes(s)) {
                if (int rc = settle_tables(s, st)) return rc;
                if (int rc = build_graphs(s)) return rc;
            }
            if (int rc = adj_segment(s, st, nf, 0)) return rc;
        }
    }
    s->adj_last_taped = true;
    s->anchor = -1;            // the taped segment does not record which buffer held the anchors
    s->adj_gen = s->gen;
    const int fin = sort_passes(s) % 2;
    CK(cudaMemcpyAsync(s->adj_fin_x, s->x[s->cur.x], N * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->adj_fin_v, s->v[s->cur.v], N * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->adj_fin_keys, s->keys[fin], N * 4, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->adj_fin_p, s->p[s->cur.p], N * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->adj_fin_col, s->col[s->cur.x], N * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->adj_fin_ids, s->ids[s->cur.x], N * 4, cudaMemcpyDeviceToDevice, st));
    if (solids) CK(cudaMemcpyAsync(s->adj_fin_w, s->w[s->cur.x], N * 4, cudaMemcpyDeviceToDevice, st));
    if (vort) CK(cudaMemcpyAsync(s->adj_fin_f, s->fext, N * 16, cudaMemcpyDeviceToDevice, st));
    s->last_stream = st;
    return PBD_OK;
}

// Make the cell tables hold the cells of `keys` (n sorted keys); `held` are the keys they hold now.
static void retable(pbd_sim* s, cudaStream_t st, const uint32_t* held, const uint32_t* keys, uint32_t n) {
    const uint32_t T = table_size(s);
    const uint32_t g = std::max(1u, std::min(div_up(n, 256), (uint32_t)s->num_sms * 8u));
    adj_clear_cells_kernel<<<g, 256, 0, st>>>(held, n, s->cell_start, T);
    adj_set_cells_kernel<<<g, 256, 0, st>>>(keys, n, s->cell_start, s->cell_end, T);
}

// The reverse pass of one segment: recompute its frames from the checkpoint already in the
// state buffers (unless the tape holds them), then walk its frames backwards, and leave the cell
// tables holding the cells of keys[fin] again.  Only enqueues work (it is recorded as a graph).
static cudaError_t enqueue_segment(pbd_sim* s, cudaStream_t st, Cur& cur, int nf, bool recompute) {
    const uint32_t N = s->N, I = s->prm.solver_iterations;
    const int fin = sort_passes(s) % 2;
    const DevParams P = make_dev_params(s);
    const bool lists = near_lists_on(s, P);
    const bool collide = s->prm.collision_type == 0;
    const uint32_t gn = div_up(N, 128), ge = div_up(N, 256);
    const bool visc_on = (s->prm.active & PBD_ACTIVE_COMPUTE_VISCOSITY) != 0;
    const uint32_t nstab = collide ? s->prm.stabilization_iterations : 0u;   // contact passes per iteration
    float4 *gx_out = s->adj_g[0], *gv_out = s->adj_g[1], *gx = s->adj_g[2];
    if (recompute) {
        for (int t = 0; t < nf; ++t) {
            uint32_t nl = 0;
            cudaError_t e = enqueue_frame(s, st, cur, false, nl, nullptr, &s->adj_tape[t]);
            if (e != cudaSuccess) return e;
        }
    }
    const uint32_t* held = s->adj_tape[nf - 1].keys;   // same contents as keys[fin]
    for (int t = nf - 1; t >= 0; --t) {
        const Tape& T = s->adj_tape[t];
        if (T.keys != held) { retable(s, st, held, T.keys, N); held = T.keys; }
        // adj_update writes all of gp: each frame starts from the same pair of buffers
        float4 *gp = s->adj_g[3], *gp2 = s->adj_g[4];
        // the frame's fixed-point scale, from the gradient entering it
        cudaMemsetAsync(s->adj_gmax, 0, 4, st);
        adj_gmax_kernel<<<ge, 256, 0, st>>>(P, gx_out, gv_out, s->adj_gmax);
        if (T.p_fin) {
            // the passes after updatePositions, last first, into gx (dL/dp final) and gp2 (dL/dv
            // before the viscosity): the viscosity's and the vorticity force's terms in one walk,
            // then omega's (dL/df of this frame's force is in gv_out, the next frame's dL/dv)
            // the frame's full list as the forward recorded it into the tape (unset when the
            // forward walked the cells: then the reverse walks them too)
            const NbList Ft = (T.full && use_full_list(s)) ? NbList{T.full, T.full_meta, N, s->fl_slots}
                                                           : NbList{nullptr, nullptr, 0u, 0u};
            adj_visc_vort_kernel<<<gn, 128, 0, st>>>(P, T.p_fin, T.p_it[0], T.v_u, T.omega, T.eta, gx_out, gv_out, T.w, gx,
                                                     gp2, s->adj_gom, s->adj_scat, s->adj_scat2, s->adj_scat3,
                                                     s->cell_start, s->cell_end, s->adj_gmax, visc_on ? 1 : 0,
                                                     T.omega ? 1 : 0, Ft);
            if (T.omega)
                adj_omega_kernel<<<gn, 128, 0, st>>>(P, T.p_fin, T.p_it[0], T.v_u, s->adj_gom, s->adj_scat3, gx, gp2,
                                                     s->adj_scat2, s->adj_scat, s->cell_start, s->cell_end, s->adj_gmax, Ft);
            adj_update_visc_kernel<<<ge, 256, 0, st>>>(P, gx, gp2, gp, s->adj_scat, s->adj_scat2, s->adj_gmax);
        } else {
            adj_update_kernel<<<ge, 256, 0, st>>>(P, gx_out, gv_out, gp, gx);
        }
        for (int it = (int)I - 1; it >= 0; --it) {
            const float4* p = T.p_it[it];
            const float4* pa = T.p_it[0];
            const NbList Lt = lists ? NbList{T.near[it], T.near_meta[it], N, kListMax} : NbList{nullptr, nullptr, 0u, 0u};
            // each pass writes every particle's own terms and scatters the partners' in fixed point;
            // the next kernel adds a particle's scattered terms in one place: the same bits
            // whatever order the atomics landed in
            // the contact passes after the first (stabilizationIterations > 1), last first, each at the
            // positions it started from; the first of them also keeps the iteration's complete final
            // gradient for the density correction's terms, applied after the last pass
            unsigned long long* sin = s->adj_scat2;
            const float4* gD = nullptr;
            for (int k = (int)nstab - 1; k >= 1; --k) {
                unsigned long long* sout = (sin == s->adj_scat2) ? s->adj_scat3 : s->adj_scat2;
                float4* gd_out = (k == (int)nstab - 1) ? s->adj_g[5] : nullptr;
                adj_collide_kernel<<<gn, 128, 0, st>>>(P, T.p_s[it][k - 1], pa, gp, gx, gp2, sin, sout, gd_out,
                                                       s->cell_start, s->cell_end, s->adj_gmax, T.w);
                std::swap(gp, gp2);
                sin = sout;
                if (gd_out) gD = gd_out;
            }
            adj_delta_kernel<<<gn, 128, 0, st>>>(P, p, pa, T.lam[it], gp, gx, gp2, s->adj_glam, s->adj_scat,
                                                 sin, s->cell_start, s->cell_end, s->adj_acc, collide && nstab > 0, Lt,
                                                 s->adj_gmax, T.w, gD);
            adj_lambda_kernel<<<gn, 128, 0, st>>>(P, p, pa, T.aux[it], s->adj_glam, gp2, s->adj_scat2, s->adj_scat,
                                                  s->cell_start, s->cell_end, s->adj_acc, Lt, s->adj_gmax);
            std::swap(gp, gp2);
        }
        adj_predict_kernel<<<ge, 256, 0, st>>>(P, T.perm, T.x_in, T.v_in, T.fext ? T.fext : s->fext, gp, gx, gx_out, gv_out,
                                               s->adj_scat2, s->adj_gmax);
    }
    // back to the tables the next recompute's predict expects: the cells of keys[fin]
    retable(s, st, held, s->keys[fin], N);
    return cudaGetLastError();
}

// Run one adjoint segment from the current buffer record as a recorded graph (recorded on first
// use and kept while the parameters, N, the block size and the workspace stay the same):
// kind 0: nf taped forward frames; 1: recompute nf taped frames, then their reverse pass;
// 2: the reverse pass of nf frames whose tape is already there.
static int adj_segment(pbd_sim* s, cudaStream_t st, int nf, int kind) {
    if (s->adj_graphs_pgen != s->pgen || s->adj_graphs_arena != s->adj_arena || s->adj_graphs.size() >= 16) {
        CK(cudaStreamSynchronize(st));
        for (auto& g : s->adj_graphs) cudaGraphExecDestroy(g.exec);
        s->adj_graphs.clear();
        s->adj_graphs_pgen = s->pgen;
        s->adj_graphs_arena = s->adj_arena;
    }
    pbd_sim::AdjGraph* g = nullptr;
    for (auto& h : s->adj_graphs)
        if (h.start == s->cur && h.nf == nf && h.kind == kind) { g = &h; break; }
    if (!g) {
        pbd_sim::AdjGraph h{s->cur, nf, kind, s->cur, nullptr};
        CK(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        if (kind == 0) {
            for (int t = 0; t < nf && e == cudaSuccess; ++t) {
                uint32_t nl = 0;
                e = enqueue_frame(s, s->cap_stream, h.end, false, nl, nullptr, &s->adj_tape[t]);
            }
        } else {
            e = enqueue_segment(s, s->cap_stream, h.end, nf, kind == 1);
        }
        cudaGraph_t graph = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(s->cap_stream, &graph);
        if (e != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return cuda_fail("adjoint segment capture", e); }
        if (e2 != cudaSuccess) return cuda_fail("cudaStreamEndCapture", e2);
        e = cudaGraphInstantiate(&h.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_fail("cudaGraphInstantiate", e);
        s->adj_graphs.push_back(h);
        g = &s->adj_graphs.back();
    }
    CK(cudaGraphLaunch(g->exec, st));
    s->cur = g->end;
    s->table_hint = s->N;
    return PBD_OK;
}

int pbd_adjoint_backward(pbd_sim* s, const float* dL_dx_final, float* dL_dv0, float* dL_dx0, double* dL_drho0,
                         double* dL_deps, void* stream) {
    clear_error();
    if (int rc = check_sim(s, "pbd_adjoint_backward")) return rc;
    if (!s->adj_arena || s->adj_steps == 0) { set_error("pbd_adjoint_backward: run pbd_adjoint_forward first"); return PBD_ERR_INVALID_ARG; }
    if (s->N != s->adj_n || s->gen != s->adj_gen) { set_error("pbd_adjoint_backward: the state or the parameters changed since pbd_adjoint_forward"); return PBD_ERR_INVALID_ARG; }
    if (!dL_dx_final) { set_error("pbd_adjoint_backward: null dL/dx"); return PBD_ERR_INVALID_ARG; }
    if (int rc = adjoint_supported(s)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (s->last_stream != st) CK(cudaStreamSynchronize(s->last_stream));
    const uint32_t N = s->N;
    const int fin = sort_passes(s) % 2;
    float4 *gx_out = s->adj_g[0], *gv_out = s->adj_g[1];
    CK(cudaMemcpyAsync(gx_out, dL_dx_final, (size_t)N * 16, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(gv_out, 0, (size_t)N * 16, st));
    const uint32_t nblk = div_up(N, 128);   // the reverse kernels' blocks: two accumulators each
    CK(cudaMemsetAsync(s->adj_acc, 0, (size_t)nblk * 16, st));
    CK(cudaMemsetAsync(s->adj_scat, 0, (size_t)N * 32, st));
    CK(cudaMemsetAsync(s->adj_scat2, 0, (size_t)N * 32, st));
    for (int ck = s->adj_nck - 1; ck >= 0; --ck) {
        const int f0 = ck * s->adj_every;
        const int nf = std::min(s->adj_every, s->adj_steps - f0);
        const bool recompute = ck + 1 < s->adj_nck || !s->adj_last_taped;
        if (recompute) {   // the segment's checkpoint into the state buffers
            CK(cudaMemcpyAsync(s->x[s->cur.x], s->adj_ck_x + (size_t)ck * N, (size_t)N * 16, cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(s->v[s->cur.v], s->adj_ck_v + (size_t)ck * N, (size_t)N * 16, cudaMemcpyDeviceToDevice, st));
            if (s->adj_ck_w)
                CK(cudaMemcpyAsync(s->w[s->cur.x], s->adj_ck_w + (size_t)ck * N, (size_t)N * 4, cudaMemcpyDeviceToDevice, st));
            if (s->adj_ck_f)
                CK(cudaMemcpyAsync(s->fext, s->adj_ck_f + (size_t)ck * N, (size_t)N * 16, cudaMemcpyDeviceToDevice, st));
        }
        if (int rc = adj_segment(s, st, nf, recompute ? 1 : 2)) return rc;
    }
    // restore the state after the forward: tables, sorted keys, x, v, p, colours and ids
    retable(s, st, s->keys[fin], s->adj_fin_keys, N);
    CK(cudaMemcpyAsync(s->keys[fin], s->adj_fin_keys, (size_t)N * 4, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->x[s->cur.x], s->adj_fin_x, (size_t)N * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->v[s->cur.v], s->adj_fin_v, (size_t)N * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->p[s->cur.p], s->adj_fin_p, (size_t)N * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->col[s->cur.x], s->adj_fin_col, (size_t)N * 16, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->ids[s->cur.x], s->adj_fin_ids, (size_t)N * 4, cudaMemcpyDeviceToDevice, st));
    if (s->adj_fin_w) CK(cudaMemcpyAsync(s->w[s->cur.x], s->adj_fin_w, (size_t)N * 4, cudaMemcpyDeviceToDevice, st));
    if (s->adj_fin_f) CK(cudaMemcpyAsync(s->fext, s->adj_fin_f, (size_t)N * 16, cudaMemcpyDeviceToDevice, st));
    s->adj_last_taped = s->adj_nck == 1;       // else the tape now holds the first segment
    s->anchor = -1;
    std::vector<double> acc((size_t)nblk * 2);
    CK(cudaMemcpyAsync(acc.data(), s->adj_acc, (size_t)nblk * 16, cudaMemcpyDeviceToHost, st));
    if (dL_dv0) CK(cudaMemcpyAsync(dL_dv0, gv_out, (size_t)N * 16, cudaMemcpyDeviceToHost, st));
    if (dL_dx0) CK(cudaMemcpyAsync(dL_dx0, gx_out, (size_t)N * 16, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double drho = 0.0, deps = 0.0;   // the blocks' slots in index order
    for (uint32_t b = 0; b < nblk; ++b) { drho += acc[2 * (size_t)b]; deps += acc[2 * (size_t)b + 1]; }
    if (dL_drho0) *dL_drho0 = drho;
    if (dL_deps) *dL_deps = deps;
    s->last_stream = st;
    return PBD_OK;
}
}  // extern "C"
