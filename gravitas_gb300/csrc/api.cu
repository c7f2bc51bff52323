// api.cu — the C-ABI of include/gbh.h: contexts, grow-only device buffers, and the host side
// of the force and step path (bh.Solver.Accelerations, Simulation.Step) over the kernels of
// tree.cu and walk.cu.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbh_internal.cuh"

using gbh::DevInfo;
using gbh::Launch;

// One KDK step captured as a CUDA graph, valid for the sizes, parameters and buffers it was
// captured with.
struct StepGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t stage_nodes[3] = {};  // event-record nodes: build start, walk start, walk end
    int64_t launches = 0;                 // kernels in one replay
    // validity key
    int64_t n = -1, tree_gen = -1, state_gen = -1, sys_gen = -1;
    gbh_params p = {};
    double dt = 0;
    const void *kind = nullptr, *alive = nullptr;
};

struct gbh_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // device-to-host copies that overlap the walk
    cudaEvent_t copy_done = nullptr;
    cudaEvent_t ev[6] = {};
    gbh::TreeBufs tb;
    // resident state (state order)
    int64_t cap = 0, n = 0;
    int64_t state_gen = 0;  // incremented whenever the state buffers are reallocated
    // forest: systems of the resident state (nsys == 1: a plain state)
    int32_t nsys = 1;
    int64_t sys_gen = 0;      // incremented whenever the systems change
    uint16_t *sys_of = nullptr;
    int64_t sys_of_cap = 0;
    int64_t *sys_off = nullptr;
    int64_t sys_off_cap = 0;
    bool have_state = false, acc_valid = false;
    int32_t state_holes = 0;
    bool state_has_kind = false, state_has_alive = false;
    double *px = nullptr, *py = nullptr, *pz = nullptr, *vx = nullptr, *vy = nullptr, *vz = nullptr;
    double *ax = nullptr, *ay = nullptr, *az = nullptr, *mass = nullptr;
    uint8_t *kind = nullptr, *alive = nullptr;
    // scratch of the potential and direct-sum calls
    double *part = nullptr;
    int64_t part_cap = 0;
    double *scalar = nullptr;
    int32_t *holes = nullptr;
    int64_t holes_cap = 0;
    int64_t *targets = nullptr;
    double *tout = nullptr;
    int64_t targets_cap = 0;
    float *probe = nullptr;
    double *scratch3 = nullptr;  // 3 x n doubles the diagnostics' tree build may write
    int64_t scratch3_cap = 0;
    uint8_t *rung = nullptr;     // block steps: rung and step-end tick per body
    int64_t rung_cap = 0;
    int32_t *end_tick = nullptr;
    int64_t end_cap = 0;
    // per-stage events of the current call: (build start, walk start, walk end) triples
    std::vector<cudaEvent_t> evpool;
    size_t evused = 0;
    StepGraph step_graph;
    gbh::AdjTape adj;  // tape of gbh_fwd_save
    gbh::SplitBufs split;             // buffers of the hole-aware step
    std::vector<int32_t> hole_list;   // alive holes of the resident state, ascending
    bool use_graphs = true;
    bool use_lpt = true;  // longest-first group order of the mixed walk
    bool use_split = true;  // split walks of few groups over several warps
    bool use_paired = false;  // 64-star groups always take the paired walk
    int64_t active_hint = 0;  // block steps: the stars the last event walked
    cudaEvent_t wait_ev = nullptr;  // GBH_CFG_BLOCKING_SYNC: host waits sleep on this event
    cudaEvent_t ahead[4] = {};      // GBH_CFG_BLOCKING_SYNC: ends of the last steps launched
    bool capturing = false;  // stage events become graph event-record nodes
    // The corrupt-link test hook: with GBH_FAULT_LINK set (non-empty) when the context is created,
    // the next tree built outside graph capture gets a cycle (the last leaf's skip link points back
    // at node 0) before its walk, so the walk runs into its step bound and the call returns
    // GBH_ERR_LIMIT naming the walk kernel. It fires once.
    bool fault_link = false;
    // bookkeeping
    int64_t launches = 0;
    int64_t h2d = 0, d2h = 0;
    int64_t last_substeps = 1;  // substeps of the last hole-aware step
    DevInfo info_host = {};
    gbh_timings last = {};
    std::string err;
};

namespace gbh {

// NVTX range for profilers (Nsight Systems shows every C-ABI call and its build and walk stages
// on the CPU timeline); without a profiler attached a push or pop is a no-op call.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// The allocation-failure test hook: -1 disarmed, k >= 0 fails the allocation after k more.
static std::atomic<long long> g_alloc_fault{-1};

void arm_alloc_fault(long long after) { g_alloc_fault.store(after < 0 ? -1 : after); }

cudaError_t dev_alloc_bytes(void **p, size_t bytes) {
    long long k = g_alloc_fault.load();
    while (k >= 0) {
        if (g_alloc_fault.compare_exchange_weak(k, k - 1)) {
            if (k == 0) {  // fire once; the counter is now -1 (disarmed)
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    return cudaMalloc(p, bytes);
}

}  // namespace gbh

namespace {

int fail(gbh_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? GBH_ERR_NOMEM : GBH_ERR_CUDA, "%s: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);                       \
    } while (0)

template <class T>
cudaError_t grow(T *&p, int64_t &cap, int64_t need) {
    if (need <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    int64_t c = std::max<int64_t>(need + need / 4, 16);
    cudaError_t e = gbh::dev_alloc(&p, sizeof(T) * size_t(c));
    cap = e == cudaSuccess ? c : 0;
    return e;
}

// Grow-only target list and its 3-column output (tout holds 3 x targets_cap doubles).
cudaError_t grow_targets(gbh_ctx *c, int64_t need) {
    if (need <= c->targets_cap && c->targets && c->tout) return cudaSuccess;
    int64_t cap = 0;
    cudaError_t e = grow(c->targets, cap, need);
    if (e != cudaSuccess) {
        c->targets_cap = 0;
        return e;
    }
    if (c->tout) cudaFree(c->tout);
    c->tout = nullptr;
    e = gbh::dev_alloc(&c->tout, sizeof(double) * 3 * size_t(cap));
    c->targets_cap = e == cudaSuccess ? cap : 0;
    return e;
}

void free_state(gbh_ctx *c) {
    void *ptrs[] = {c->px, c->py, c->pz, c->vx, c->vy, c->vz, c->ax, c->ay, c->az, c->mass, c->kind, c->alive};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    c->px = c->py = c->pz = c->vx = c->vy = c->vz = c->ax = c->ay = c->az = c->mass = nullptr;
    c->kind = c->alive = nullptr;
    c->cap = 0;
}

cudaError_t ensure_state(gbh_ctx *c, int64_t n) {
    if (n <= c->cap && c->px) return cudaSuccess;
    free_state(c);
    int64_t cap = std::max<int64_t>(n + n / 4, 16);
    cudaError_t e = cudaSuccess;
    double **d[] = {&c->px, &c->py, &c->pz, &c->vx, &c->vy, &c->vz, &c->ax, &c->ay, &c->az, &c->mass};
    for (double **p : d)
        if (e == cudaSuccess) e = gbh::dev_alloc(p, sizeof(double) * size_t(cap));
    if (e == cudaSuccess) e = gbh::dev_alloc(&c->kind, size_t(cap));
    if (e == cudaSuccess) e = gbh::dev_alloc(&c->alive, size_t(cap));
    if (e != cudaSuccess) {
        free_state(c);
        return e;
    }
    c->cap = cap;
    ++c->state_gen;
    return cudaSuccess;
}

int check_params(gbh_ctx *ctx, const gbh_params *p) {
    if (!p) return fail(ctx, GBH_ERR_ARG, "params is NULL");
    if (!(p->theta >= 0 && p->theta <= 1)) return fail(ctx, GBH_ERR_ARG, "theta %g outside [0, 1]", p->theta);
    if (!(p->softening >= 0)) return fail(ctx, GBH_ERR_ARG, "softening %g < 0", p->softening);
    if (p->leaf_size < 0 || p->leaf_size > 1 << 20) return fail(ctx, GBH_ERR_ARG, "leaf_size %d", p->leaf_size);
    if (p->walk < GBH_WALK_MIXED || p->walk > GBH_WALK_FP64) return fail(ctx, GBH_ERR_ARG, "walk %d", p->walk);
    if (p->group_size != 0 && p->group_size != 32 && p->group_size != 64)
        return fail(ctx, GBH_ERR_ARG, "group_size %d (0, 32 or 64)", p->group_size);
    if (p->list_depth != 0 && (p->list_depth < 2 || p->list_depth > gbh::list_depth_max(false)))
        return fail(ctx, GBH_ERR_ARG, "list_depth %d (0, or 2 to %d)", p->list_depth, gbh::list_depth_max(false));
    if (!(p->c >= 0 && std::isfinite(p->c))) return fail(ctx, GBH_ERR_ARG, "c %g must be finite and >= 0", p->c);
    return GBH_OK;
}

double theta_of(const gbh_params *p) { return p->theta == 0 ? 0.9 : p->theta; }  // bh.go:69-74

// Stars per group of the mixed walk: 32 (the list walk, one star a lane) or 64 (the list walk with
// two, or for a single system with so few groups per SM that the paired walk shares each group
// among several warps, that walk). By default 64 for forests and large single systems (two stars
// a lane: 0.93x the walk time of one on the 1M merger, and the autotuner's pick on the 64-system
// forest) and for small ones (split walks), else 32.
int group_of(const gbh_params *p, int64_t n, bool forest) {
    if (p->group_size == 32 || p->group_size == 64) return p->group_size;
    if (forest) return 64;
    // 32-star groups below 2^19 bodies: the list walk, shared among warps when the groups are few
    // (measured on Plummer spheres and galaxies of 16k-131k bodies, walk time against 64-star
    // groups in the paired walk's split mode: 0.11 / 0.17 ms at 16k, 0.38 / 0.76 at 65k, 0.69 /
    // 1.54 at 131k; even at 262k); above, 64-star groups (two stars a lane)
    return n >= (int64_t(1) << 19) ? 64 : 32;
}
int leaf_of(const gbh_params *p) { return p->leaf_size > 0 ? p->leaf_size : 24; }  // bh.go:17-19

int begin(gbh_ctx *ctx) {
    if (!ctx) return GBH_ERR_ARG;
    ctx->err.clear();
    ctx->evused = 0;
    ctx->launches = 0;
    ctx->h2d = ctx->d2h = 0;
    ctx->last = gbh_timings{};
    cudaError_t e = cudaSetDevice(ctx->device);  // cgo callers may migrate between OS threads
    if (e != cudaSuccess) return fail(ctx, GBH_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    return GBH_OK;
}

Launch launch_of(gbh_ctx *ctx) { return Launch{ctx->stream, &ctx->launches, ctx->num_sms}; }

// Waits for the context's stream: a spin in the CUDA driver by default, a sleep on a blocking-sync
// event with GBH_CFG_BLOCKING_SYNC (the waiting thread then leaves its core to other work).
cudaError_t wait_stream(gbh_ctx *ctx) {
    if (!ctx->wait_ev) return cudaStreamSynchronize(ctx->stream);
    cudaError_t e = cudaEventRecord(ctx->wait_ev, ctx->stream);
    return e != cudaSuccess ? e : cudaEventSynchronize(ctx->wait_ev);
}

// Before launching step s: with GBH_CFG_BLOCKING_SYNC, sleep until step s - 4 has finished, so
// that the CUDA driver's launch queue never fills (a full queue makes the launching thread spin).
cudaError_t throttle_before(gbh_ctx *ctx, int64_t s) {
    if (!ctx->wait_ev || s < 4) return cudaSuccess;
    return cudaEventSynchronize(ctx->ahead[s % 4]);
}

cudaError_t throttle_after(gbh_ctx *ctx, int64_t s) {
    return ctx->wait_ev ? cudaEventRecord(ctx->ahead[s % 4], ctx->stream) : cudaSuccess;
}

// Takes the next stage event of the call from the context's event pool (creating it if needed).
cudaError_t next_stage_event(gbh_ctx *ctx, cudaEvent_t *ev) {
    if (ctx->evused == ctx->evpool.size()) {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
        ctx->evpool.push_back(e);
    }
    *ev = ctx->evpool[ctx->evused++];
    return cudaSuccess;
}

// Records the next stage event of the call on the context's stream.
cudaError_t stage_event(gbh_ctx *ctx) {
    cudaEvent_t ev;
    cudaError_t r = next_stage_event(ctx, &ev);
    if (r != cudaSuccess) return r;
    return ctx->capturing ? cudaEventRecordWithFlags(ev, ctx->stream, cudaEventRecordExternal)
                          : cudaEventRecord(ev, ctx->stream);
}

int h2d(gbh_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (!bytes) return GBH_OK;
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    ctx->h2d += int64_t(bytes);
    return GBH_OK;
}

int d2h(gbh_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (!bytes) return GBH_OK;
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->d2h += int64_t(bytes);
    return GBH_OK;
}

// Tree build + walk on device arrays; accelerations of alive non-hole bodies, holes zeroed.
// forest: the resident state's systems (each its own tree) instead of one system.
int forces(gbh_ctx *ctx, const gbh_params *p, int64_t n, const double *px, const double *py, const double *pz,
           const double *mass, const uint8_t *kind, const uint8_t *alive, double *ax, double *ay, double *az,
           double theta, bool forest = false) {
    Launch L = launch_of(ctx);
    int leaf = leaf_of(p);
    forest = forest && ctx->nsys > 1;
    CK(gbh::tree_alloc(ctx->tb, n, leaf, forest ? ctx->nsys : 1));
    ctx->tb.group = group_of(p, n, forest);
    ctx->tb.list_depth = p->list_depth;
    ctx->tb.lpt = ctx->use_lpt;
    ctx->tb.split = ctx->use_split;
    ctx->tb.paired = ctx->use_paired;
    ctx->tb.walk_hint = 0;
    CK(stage_event(ctx));
    {
        gbh::NvtxRange r("tree build");
        CK(gbh::tree_build(L, ctx->tb, n, px, py, pz, mass, kind, alive, ax, ay, az, theta, leaf,
                           p->dark_matter_off, p->walk == GBH_WALK_FP64, p->walk == GBH_WALK_PLAIN,
                           forest ? ctx->sys_of : nullptr, forest ? ctx->sys_off : nullptr));
    }
    if (ctx->fault_link && !ctx->capturing) {
        ctx->fault_link = false;
        CK(gbh::fault_link(L, ctx->tb));
    }
    CK(stage_event(ctx));
    gbh::NvtxRange walk_range("walk");
    double eps2 = p->softening * p->softening;
    int quad = !p->monopole_only;
    switch (p->walk) {
        case GBH_WALK_FP64:
            CK(gbh::walk_fp64(L, ctx->tb, n, eps2, quad, ax, ay, az));
            break;
        case GBH_WALK_PLAIN:
            if (!quad) return fail(ctx, GBH_ERR_ARG, "the plain FP32 walk always uses quadrupoles (as the Metal kernel)");
            CK(gbh::walk_plain(L, ctx->tb, ctx->tb.cap_n, float(eps2), ax, ay, az));
            break;
        default:
            // sized by the body count (not the capacity): a split walk's parts depend on n alone
            CK(gbh::walk_mixed(L, ctx->tb, n, float(eps2), quad, ax, ay, az));
            break;
    }
    CK(stage_event(ctx));
    return GBH_OK;
}

// The status of a device-side check recorded in the DevInfo the host has read back.
int info_status(gbh_ctx *ctx) {
    const DevInfo &i = ctx->info_host;
    if (!i.err) return GBH_OK;
    if (i.err_where == gbh::kErrNonFinite)
        return fail(ctx, GBH_ERR_ARG, "an alive star has a non-finite position or mass (outputs are undefined)");
    return fail(ctx, GBH_ERR_LIMIT, "device walk exceeded its step bound (kernel %d)", i.err_where);
}

// Waits for the stream, reads the device scalars and fills the timings of the call.
int finish(gbh_ctx *ctx, bool tree) {
    CK(cudaEventRecord(ctx->ev[5], ctx->stream));
    if (tree && ctx->tb.info) {
        CK(cudaMemcpyAsync(&ctx->info_host, ctx->tb.info, sizeof(DevInfo), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(wait_stream(ctx));
    float ms = 0;
    gbh_timings &t = ctx->last;
    if (cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[5]) == cudaSuccess) t.total_ms = ms;
    for (size_t k = 0; k + 2 < ctx->evused; k += 3) {
        if (cudaEventElapsedTime(&ms, ctx->evpool[k], ctx->evpool[k + 1]) == cudaSuccess) t.build_ms += ms;
        if (cudaEventElapsedTime(&ms, ctx->evpool[k + 1], ctx->evpool[k + 2]) == cudaSuccess) t.walk_ms += ms;
    }
    t.step_ms = t.total_ms - t.build_ms - t.walk_ms;
    t.launches = ctx->launches;
    t.substeps = ctx->last_substeps;
    t.h2d_bytes = ctx->h2d;
    t.d2h_bytes = ctx->d2h;
    if (tree) {
        t.nstars = ctx->info_host.nstars;
        t.nnodes = ctx->info_host.nnodes;
        return info_status(ctx);
    }
    return GBH_OK;
}

// Alive holes among n bodies. memchr (vectorised in the C library) skips the runs of other kinds,
// so a host call on a million bodies costs tens of microseconds, not a byte loop.
int count_holes(const uint8_t *kind, const uint8_t *alive, int64_t n) {
    if (!kind || n <= 0) return 0;
    int64_t h = 0;
    for (const uint8_t *q = kind, *end = kind + n;
         (q = static_cast<const uint8_t *>(std::memchr(q, GBH_BLACK_HOLE, size_t(end - q)))) != nullptr; ++q)
        if (!alive || alive[q - kind]) ++h;
    return int(std::min<int64_t>(h, 1 << 30));
}

void free_graph(StepGraph &g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
    g = StepGraph{};
}

bool same_params(const gbh_params &a, const gbh_params &b) {
    return a.theta == b.theta && a.softening == b.softening && a.leaf_size == b.leaf_size &&
           a.monopole_only == b.monopole_only && a.dark_matter_off == b.dark_matter_off && a.walk == b.walk &&
           a.group_size == b.group_size && a.list_depth == b.list_depth && a.c == b.c;
}

// out[q] = a[idx[q]] for the three arrays of a (n doubles apart in out).
__global__ void k_gather3(int64_t cnt, const int64_t *__restrict__ idx, const double *__restrict__ ax,
                          const double *__restrict__ ay, const double *__restrict__ az, double *out) {
    int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (q >= cnt) return;
    int64_t i = idx[q];
    out[q] = ax[i];
    out[cnt + q] = ay[i];
    out[2 * cnt + q] = az[i];
}

// Captures one resident step (kick + drift, forces, kick) into ctx->step_graph.
int capture_step(gbh_ctx *ctx, const gbh_params *p, double dt, const uint8_t *kind, const uint8_t *alive) {
    StepGraph &g = ctx->step_graph;
    free_graph(g);
    Launch L = launch_of(ctx);
    const int64_t n = ctx->n;
    const double h = 0.5 * dt;
    const size_t ev0 = ctx->evused;
    const int64_t l0 = ctx->launches;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->capturing = true;
    int rc = GBH_OK;
    cudaError_t e = gbh::kick_drift(L, n, h, dt, p->c, ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy, ctx->vz, ctx->ax, ctx->ay,
                                    ctx->az);
    if (e == cudaSuccess)
        rc = forces(ctx, p, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind, alive, ctx->ax, ctx->ay, ctx->az,
                    theta_of(p), true);
    if (e == cudaSuccess && rc == GBH_OK) e = gbh::kick(L, n, h, ctx->vx, ctx->vy, ctx->vz, ctx->ax, ctx->ay, ctx->az);
    cudaGraph_t graph = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
    ctx->capturing = false;
    if (e != cudaSuccess || rc != GBH_OK || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (rc != GBH_OK) return rc;
        return fail(ctx, GBH_ERR_CUDA, "step capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    g.graph = graph;
    g.launches = ctx->launches - l0;
    ctx->launches = l0;
    // the event-record nodes of the three stage events recorded by forces()
    size_t count = 0;
    CK(cudaGraphGetNodes(graph, nullptr, &count));
    std::vector<cudaGraphNode_t> nodes(count);
    CK(cudaGraphGetNodes(graph, nodes.data(), &count));
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        CK(cudaGraphNodeGetType(nd, &t));
        if (t != cudaGraphNodeTypeEventRecord) continue;
        cudaEvent_t ev;
        CK(cudaGraphEventRecordNodeGetEvent(nd, &ev));
        for (int k = 0; k < 3; ++k)
            if (ev == ctx->evpool[ev0 + k]) g.stage_nodes[k] = nd;
    }
    ctx->evused = ev0;  // the captured events were placeholders; replays get their own
    for (auto nd : g.stage_nodes)
        if (!nd) return fail(ctx, GBH_ERR_CUDA, "step capture: stage events not found in the graph");
    CK(cudaGraphInstantiate(&g.exec, graph, 0));
    g.n = n;
    g.p = *p;
    g.dt = dt;
    g.tree_gen = ctx->tb.generation;
    g.state_gen = ctx->state_gen;
    g.sys_gen = ctx->sys_gen;
    g.kind = kind;
    g.alive = alive;
    return GBH_OK;
}

// Steps on the resident state (sim.go:252-288, no holes, no hydro).
// The hole-aware step (split.go:162-200, stepSplit) without gas, instant gravity and no spins:
// forces of pairs with a hole summed directly (Paczynski-Wiita star-hole pairs for c > 0), near
// stars and holes in power-of-two substeps, star-star forces from the tree once per step. The substep count of the last step goes to ctx->last_substeps.
int run_split_steps(gbh_ctx *ctx, const gbh_params *p, double dt, int64_t nsteps) {
    Launch L = launch_of(ctx);
    const int64_t n = ctx->n;
    const uint8_t *kind = ctx->kind;  // holes imply kinds
    const uint8_t *alive = ctx->state_has_alive ? ctx->alive : nullptr;
    const double theta = theta_of(p), eps2 = p->softening * p->softening, h = 0.5 * dt;
    const int dm = p->dark_matter_off;
    const double c = p->c;
    gbh::SplitBufs &sb = ctx->split;
    CK(gbh::split_reserve(sb, n, ctx->hole_list));
    CK(cudaMemcpyAsync(sb.holes, ctx->hole_list.data(), sizeof(int32_t) * ctx->hole_list.size(),
                       cudaMemcpyHostToDevice, ctx->stream));
    double *px = ctx->px, *py = ctx->py, *pz = ctx->pz, *vx = ctx->vx, *vy = ctx->vy, *vz = ctx->vz;
    auto slow = [&]() {  // Solver.Accelerations: star-star forces, holes get 0
        return forces(ctx, p, n, px, py, pz, ctx->mass, kind, alive, ctx->ax, ctx->ay, ctx->az, theta, false);
    };
    if (!ctx->acc_valid) {  // initForces (gas.go:14-17)
        int rc = slow();
        if (rc) return rc;
        ctx->acc_valid = true;
    }
    unsigned long long sc[2];
    for (int64_t step = 0; step < nsteps; ++step) {
        // classify (split.go:39-85): the host needs the substep count
        CK(gbh::split_classify(L, sb, n, px, py, pz, ctx->mass, kind, eps2, c, 20.0 * dt));
        CK(cudaMemcpyAsync(sc, sb.scalars, sizeof sc, cudaMemcpyDeviceToHost, ctx->stream));
        CK(wait_stream(ctx));
        double tau_min;
        std::memcpy(&tau_min, &sc[0], sizeof tau_min);
        const int32_t nnear = int32_t(sc[1]);
        int64_t k = 1;
        if (!std::isinf(tau_min))
            while (double(k) * tau_min < 20.0 * dt && k < 256) k *= 2;
        ctx->last_substeps = k;
        CK(gbh::split_outer(L, sb, n, px, py, pz, ctx->mass, kind, dm, eps2, c));
        CK(gbh::split_kick_outer(L, sb, n, h, vx, vy, vz, ctx->ax, ctx->ay, ctx->az));
        const double hs = dt / double(k);
        CK(gbh::split_fast(L, sb, n, nnear, px, py, pz, ctx->mass, kind, dm, eps2, c));
        for (int64_t q = 0; q < k; ++q) {
            CK(gbh::split_fast_update(L, sb, n, nnear, false, 0.5 * hs, c, px, py, pz, vx, vy, vz));
            CK(gbh::split_fast_update(L, sb, n, nnear, true, hs, c, px, py, pz, vx, vy, vz));
            CK(gbh::split_fast(L, sb, n, nnear, px, py, pz, ctx->mass, kind, dm, eps2, c));
            CK(gbh::split_fast_update(L, sb, n, nnear, false, 0.5 * hs, c, px, py, pz, vx, vy, vz));
        }
        CK(gbh::split_drift_far(L, sb, n, dt, c, kind, px, py, pz, vx, vy, vz));
        int rc = slow();  // advanceGas without gas (blockstep.go:129-135)
        if (rc) return rc;
        CK(gbh::split_outer(L, sb, n, px, py, pz, ctx->mass, kind, dm, eps2, c));
        CK(gbh::split_kick_outer(L, sb, n, h, vx, vy, vz, ctx->ax, ctx->ay, ctx->az));
    }
    return GBH_OK;
}

int run_steps(gbh_ctx *ctx, const gbh_params *p, double dt, int64_t nsteps) {
    Launch L = launch_of(ctx);
    int64_t n = ctx->n;
    const uint8_t *kind = ctx->state_has_kind ? ctx->kind : nullptr;
    const uint8_t *alive = ctx->state_has_alive ? ctx->alive : nullptr;
    double theta = theta_of(p);
    if (!ctx->acc_valid) {  // initForces (gas.go:14-17)
        int rc = forces(ctx, p, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind, alive, ctx->ax, ctx->ay, ctx->az, theta,
                        true);
        if (rc) return rc;
        ctx->acc_valid = true;
    }
    if (ctx->use_graphs && nsteps > 0) {
        // One captured step per replay: the ~50 kernels of a step launch as one graph.
        CK(gbh::tree_alloc(ctx->tb, n, leaf_of(p), ctx->nsys));  // any growth happens outside the capture
        StepGraph &g = ctx->step_graph;
        if (!(g.exec && g.n == n && same_params(g.p, *p) && g.dt == dt && g.tree_gen == ctx->tb.generation &&
              g.state_gen == ctx->state_gen && g.sys_gen == ctx->sys_gen && g.kind == kind && g.alive == alive)) {
            int rc = capture_step(ctx, p, dt, kind, alive);
            if (rc) return rc;
        }
        for (int64_t s = 0; s < nsteps; ++s) {
            CK(throttle_before(ctx, s));
            for (int k = 0; k < 3; ++k) {
                cudaEvent_t ev;
                CK(next_stage_event(ctx, &ev));
                CK(cudaGraphExecEventRecordNodeSetEvent(g.exec, g.stage_nodes[k], ev));
            }
            CK(cudaGraphLaunch(g.exec, ctx->stream));
            ctx->launches += g.launches;
            CK(throttle_after(ctx, s));
        }
        return GBH_OK;
    }
    double h = 0.5 * dt;
    for (int64_t s = 0; s < nsteps; ++s) {
        CK(throttle_before(ctx, s));
        CK(gbh::kick_drift(L, n, h, dt, p->c, ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy, ctx->vz, ctx->ax, ctx->ay,
                           ctx->az));
        int rc = forces(ctx, p, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind, alive, ctx->ax, ctx->ay, ctx->az, theta,
                        true);
        if (rc) return rc;
        CK(gbh::kick(L, n, h, ctx->vx, ctx->vy, ctx->vz, ctx->ax, ctx->ay, ctx->az));
        CK(throttle_after(ctx, s));
    }
    return GBH_OK;
}

// Forces on the stars whose step ends at tick (block steps): tree of all stars, walk of the
// active ones only.
int forces_active(gbh_ctx *ctx, const gbh_params *p, const uint8_t *kind, const uint8_t *alive, const int32_t *end,
                  int32_t tick) {
    Launch L = launch_of(ctx);
    int leaf = leaf_of(p);
    int64_t n = ctx->n;
    CK(gbh::tree_alloc(ctx->tb, n, leaf));
    ctx->tb.group = group_of(p, n, false);  // as the global step, so that one level is that step
    ctx->tb.list_depth = p->list_depth;
    ctx->tb.lpt = ctx->use_lpt;
    ctx->tb.split = ctx->use_split;
    ctx->tb.paired = ctx->use_paired;
    ctx->tb.walk_hint = ctx->active_hint;  // this event's list is not known on the host yet
    CK(stage_event(ctx));
    CK(gbh::tree_build(L, ctx->tb, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind, alive, ctx->ax, ctx->ay, ctx->az,
                       theta_of(p), leaf, p->dark_matter_off, p->walk == GBH_WALK_FP64, p->walk == GBH_WALK_PLAIN));
    CK(gbh::select_targets(L, ctx->tb, end, tick));
    CK(stage_event(ctx));
    double eps2 = p->softening * p->softening;
    int quad = !p->monopole_only;
    switch (p->walk) {
        case GBH_WALK_FP64:
            CK(gbh::walk_fp64(L, ctx->tb, n, eps2, quad, ctx->ax, ctx->ay, ctx->az, true));
            break;
        case GBH_WALK_PLAIN:
            if (!quad) return fail(ctx, GBH_ERR_ARG, "the plain FP32 walk always uses quadrupoles (as the Metal kernel)");
            CK(gbh::walk_plain(L, ctx->tb, ctx->tb.cap_n, float(eps2), ctx->ax, ctx->ay, ctx->az, true));
            break;
        default:
            CK(gbh::walk_mixed(L, ctx->tb, n, float(eps2), quad, ctx->ax, ctx->ay, ctx->az, true));
            break;
    }
    CK(stage_event(ctx));
    return GBH_OK;
}

// Reads the device scalars (next event tick, active count) after the work issued so far.
int read_info(gbh_ctx *ctx) {
    CK(cudaMemcpyAsync(&ctx->info_host, ctx->tb.info, sizeof(DevInfo), cudaMemcpyDeviceToHost, ctx->stream));
    CK(wait_stream(ctx));
    return info_status(ctx);
}

// Block-step KDK on the resident state (see block_open in tree.cu for the scheme).
int run_block_steps(gbh_ctx *ctx, const gbh_params *p, double T, double eta, int levels, int64_t nsteps,
                    gbh_blockstats *st) {
    Launch L = launch_of(ctx);
    const int64_t n = ctx->n;
    const uint8_t *kind = ctx->state_has_kind ? ctx->kind : nullptr;
    const uint8_t *alive = ctx->state_has_alive ? ctx->alive : nullptr;
    const int32_t ticks = 1 << (levels - 1);
    const double eps = p->softening;
    CK(grow(ctx->rung, ctx->rung_cap, n));
    CK(grow(ctx->end_tick, ctx->end_cap, n));
    if (!ctx->acc_valid) {  // initForces (gas.go:14-17)
        int rc = forces(ctx, p, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind, alive, ctx->ax, ctx->ay, ctx->az,
                        theta_of(p));
        if (rc) return rc;
        ctx->acc_valid = true;
    }
    CK(gbh::tree_alloc(ctx->tb, n, leaf_of(p)));
    int rc;
    ctx->active_hint = n;  // the first event is sized for all bodies
    for (int64_t s = 0; s < nsteps; ++s) {
        CK(gbh::block_open(L, ctx->tb, n, T, levels, eta, eps, ctx->ax, ctx->ay, ctx->az, ctx->vx, ctx->vy, ctx->vz,
                           ctx->rung, ctx->end_tick));
        if ((rc = read_info(ctx))) return rc;
        if (ctx->info_host.next_count > 0) ctx->active_hint = int64_t(ctx->info_host.next_count);
        int32_t t = 0;
        while (t < ticks) {
            int32_t tn = ctx->info_host.next_tick;
            if (tn <= t || tn > ticks) return fail(ctx, GBH_ERR_LIMIT, "block steps: next event %d after %d", tn, t);
            if (st && (st->min_substep_ticks == 0 || tn - t < st->min_substep_ticks)) st->min_substep_ticks = tn - t;
            CK(gbh::block_drift(L, n, double(tn - t) * (T / double(ticks)), p->c, ctx->px, ctx->py, ctx->pz, ctx->vx,
                                ctx->vy, ctx->vz));
            t = tn;
            if ((rc = forces_active(ctx, p, kind, alive, ctx->end_tick, t))) return rc;
            CK(gbh::block_close(L, ctx->tb, n, t, T, levels, eta, eps, ctx->ax, ctx->ay, ctx->az, ctx->vx, ctx->vy,
                                ctx->vz, ctx->rung, ctx->end_tick));
            if ((rc = read_info(ctx))) return rc;
            // the next event walks the bodies due at its tick: size its walk (split or not) by them
            if (ctx->info_host.next_count > 0) ctx->active_hint = int64_t(ctx->info_host.next_count);
            if (st) {
                st->substeps += 1;
                st->evaluations += ctx->info_host.ntargets;
            }
        }
    }
    return GBH_OK;
}

int upload_state(gbh_ctx *ctx, int64_t n, const double *px, const double *py, const double *pz, const double *vx,
                 const double *vy, const double *vz, const double *ax, const double *ay, const double *az,
                 const double *mass, const uint8_t *kind, const uint8_t *alive) {
    if (n < 0 || n > (int64_t(1) << 30)) return fail(ctx, GBH_ERR_ARG, "n = %lld out of range", (long long)n);
    if (n > 0 && (!px || !py || !pz || !vx || !vy || !vz || !mass))
        return fail(ctx, GBH_ERR_ARG, "state arrays must not be NULL");
    CK(ensure_state(ctx, n));
    size_t b = sizeof(double) * size_t(n);
    int rc;
    const double *src[] = {px, py, pz, vx, vy, vz, mass};
    double *dst[] = {ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy, ctx->vz, ctx->mass};
    for (int k = 0; k < 7; ++k)
        if ((rc = h2d(ctx, dst[k], src[k], b))) return rc;
    bool acc = ax && ay && az;
    if (acc) {
        if ((rc = h2d(ctx, ctx->ax, ax, b)) || (rc = h2d(ctx, ctx->ay, ay, b)) || (rc = h2d(ctx, ctx->az, az, b)))
            return rc;
    } else if (n > 0) {
        CK(cudaMemsetAsync(ctx->ax, 0, b, ctx->stream));
        CK(cudaMemsetAsync(ctx->ay, 0, b, ctx->stream));
        CK(cudaMemsetAsync(ctx->az, 0, b, ctx->stream));
    }
    ctx->state_has_kind = kind != nullptr;
    ctx->state_has_alive = alive != nullptr;
    if (kind && (rc = h2d(ctx, ctx->kind, kind, size_t(n)))) return rc;
    if (alive && (rc = h2d(ctx, ctx->alive, alive, size_t(n)))) return rc;
    ctx->n = n;
    ctx->have_state = true;
    ctx->acc_valid = acc;
    ctx->state_holes = count_holes(kind, alive, n);
    ctx->hole_list.clear();
    if (ctx->state_holes)  // collectHoles, sim.go:294-302 (kinds and liveness do not change in a step)
        for (const uint8_t *q = kind, *end = kind + n;
             (q = static_cast<const uint8_t *>(std::memchr(q, GBH_BLACK_HOLE, size_t(end - q)))) != nullptr; ++q)
            if (!alive || alive[q - kind]) ctx->hole_list.push_back(int32_t(q - kind));
    if (ctx->nsys != 1) {
        ctx->nsys = 1;
        ++ctx->sys_gen;
    }
    return GBH_OK;
}

int download_state(gbh_ctx *ctx, double *px, double *py, double *pz, double *vx, double *vy, double *vz, double *ax,
                   double *ay, double *az) {
    size_t b = sizeof(double) * size_t(ctx->n);
    double *dst[] = {px, py, pz, vx, vy, vz, ax, ay, az};
    const double *src[] = {ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy, ctx->vz, ctx->ax, ctx->ay, ctx->az};
    for (int k = 0; k < 9; ++k)
        if (dst[k]) {
            int rc = d2h(ctx, dst[k], src[k], b);
            if (rc) return rc;
        }
    return GBH_OK;
}

}  // namespace

extern "C" {

int gbh_create(const gbh_config *cfg, gbh_ctx **out, char *err, int errlen) {
    auto report = [&](int code, const char *msg) {
        if (err && errlen > 0) {
            std::strncpy(err, msg, size_t(errlen) - 1);
            err[errlen - 1] = 0;
        }
        return code;
    };
    if (!out) return report(GBH_ERR_ARG, "out is NULL");
    *out = nullptr;
    {  // the allocation-failure test hook (see dev_alloc): armed by GBH_FAULT_ALLOC, else off
        const char *f = std::getenv("GBH_FAULT_ALLOC");
        gbh::arm_alloc_fault(f && *f ? std::atoll(f) : -1);
    }
    int dev = cfg ? cfg->device : 0;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return report(GBH_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= count) return report(GBH_ERR_ARG, "no such CUDA device");
    if ((e = cudaSetDevice(dev)) != cudaSuccess) return report(GBH_ERR_CUDA, cudaGetErrorString(e));
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, dev)) != cudaSuccess) return report(GBH_ERR_CUDA, cudaGetErrorString(e));
    if (prop.major < 10) return report(GBH_ERR_UNSUPPORTED, "libgbh is built for sm_103a (GB300)");
    gbh_ctx *c = new gbh_ctx();
    c->device = dev;
    c->use_graphs = !(cfg && (cfg->flags & GBH_CFG_NO_GRAPHS));
    c->use_lpt = !(cfg && (cfg->flags & GBH_CFG_NO_LPT));
    c->use_split = !(cfg && (cfg->flags & GBH_CFG_NO_SPLIT));
    c->use_paired = cfg && (cfg->flags & GBH_CFG_PAIRED);
    {
        const char *f = std::getenv("GBH_FAULT_LINK");
        c->fault_link = f && *f;
    }
    if (cfg && (cfg->flags & GBH_CFG_BLOCKING_SYNC)) {
        e = cudaEventCreateWithFlags(&c->wait_ev, cudaEventBlockingSync | cudaEventDisableTiming);
        for (auto &ev : c->ahead)
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventBlockingSync | cudaEventDisableTiming);
        if (e != cudaSuccess) {
            gbh_destroy(c);
            return report(GBH_ERR_CUDA, cudaGetErrorString(e));
        }
    }
    c->num_sms = prop.multiProcessorCount;
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete c;
        return report(GBH_ERR_CUDA, cudaGetErrorString(e));
    }
    for (auto &ev : c->ev) {
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) {
            gbh_destroy(c);
            return report(GBH_ERR_CUDA, cudaGetErrorString(e));
        }
    }
    if ((e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&c->copy_done, cudaEventDisableTiming)) != cudaSuccess) {
        gbh_destroy(c);
        return report(GBH_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = c;
    return report(GBH_OK, "");
}

void gbh_destroy(gbh_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_graph(c->step_graph);
    gbh::tree_free(c->tb);
    gbh::adj_free(c->adj);
    gbh::split_free(c->split);
    free_state(c);
    void *ptrs[] = {c->part,  c->scalar,   c->holes, c->targets,  c->tout,   c->probe,
                    c->scratch3, c->rung, c->end_tick, c->sys_of, c->sys_off};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto &ev : c->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto &ev : c->evpool) cudaEventDestroy(ev);
    if (c->wait_ev) cudaEventDestroy(c->wait_ev);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->copy_done) cudaEventDestroy(c->copy_done);
    for (auto &ev : c->ahead)
        if (ev) cudaEventDestroy(ev);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char *gbh_last_error(const gbh_ctx *ctx) { return ctx ? ctx->err.c_str() : "NULL context"; }

int gbh_device_name(gbh_ctx *ctx, char *out, int len) {
    int rc = begin(ctx);
    if (rc) return rc;
    if (!out || len <= 0) return fail(ctx, GBH_ERR_ARG, "bad output buffer");
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, ctx->device));
    std::strncpy(out, prop.name, size_t(len) - 1);
    out[len - 1] = 0;
    return GBH_OK;
}

int gbh_accelerations(gbh_ctx *ctx, const gbh_params *p, int64_t n, const double *px, const double *py,
                      const double *pz, const double *mass, const uint8_t *kind, const uint8_t *alive, double *ax,
                      double *ay, double *az) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc || (rc = check_params(ctx, p))) return rc;
    if (n < 0 || n > (int64_t(1) << 30)) return fail(ctx, GBH_ERR_ARG, "n = %lld out of range", (long long)n);
    if (n == 0) return GBH_OK;
    if (!px || !py || !pz || !mass || !ax || !ay || !az) return fail(ctx, GBH_ERR_ARG, "array argument is NULL");
    CK(ensure_state(ctx, n));
    ctx->have_state = false;  // the state buffers now hold this call's arrays
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    size_t b = sizeof(double) * size_t(n);
    if ((rc = h2d(ctx, ctx->px, px, b)) || (rc = h2d(ctx, ctx->py, py, b)) || (rc = h2d(ctx, ctx->pz, pz, b)) ||
        (rc = h2d(ctx, ctx->mass, mass, b)))
        return rc;
    // Dead bodies keep their entries (bh.go:92-101 writes only stars and holes).
    if ((rc = h2d(ctx, ctx->ax, ax, b)) || (rc = h2d(ctx, ctx->ay, ay, b)) || (rc = h2d(ctx, ctx->az, az, b))) return rc;
    if (kind && (rc = h2d(ctx, ctx->kind, kind, size_t(n)))) return rc;
    if (alive && (rc = h2d(ctx, ctx->alive, alive, size_t(n)))) return rc;
    rc = forces(ctx, p, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind ? ctx->kind : nullptr,
                alive ? ctx->alive : nullptr, ctx->ax, ctx->ay, ctx->az, theta_of(p));
    if (rc) return rc;
    if ((rc = d2h(ctx, ax, ctx->ax, b)) || (rc = d2h(ctx, ay, ctx->ay, b)) || (rc = d2h(ctx, az, ctx->az, b))) return rc;
    return finish(ctx, true);
}

int gbh_potential_energy(gbh_ctx *ctx, const gbh_params *p, int64_t n, const double *px, const double *py,
                         const double *pz, const double *mass, const uint8_t *kind, const uint8_t *alive, double c,
                         double *u) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc || (rc = check_params(ctx, p))) return rc;
    if (!u) return fail(ctx, GBH_ERR_ARG, "u is NULL");
    *u = 0;
    if (n < 0 || n > (int64_t(1) << 30)) return fail(ctx, GBH_ERR_ARG, "n out of range");
    if (n == 0) return GBH_OK;
    if (!px || !py || !pz || !mass) return fail(ctx, GBH_ERR_ARG, "array argument is NULL");
    CK(ensure_state(ctx, n));
    ctx->have_state = false;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    size_t b = sizeof(double) * size_t(n);
    if ((rc = h2d(ctx, ctx->px, px, b)) || (rc = h2d(ctx, ctx->py, py, b)) || (rc = h2d(ctx, ctx->pz, pz, b)) ||
        (rc = h2d(ctx, ctx->mass, mass, b)))
        return rc;
    if (kind && (rc = h2d(ctx, ctx->kind, kind, size_t(n)))) return rc;
    if (alive && (rc = h2d(ctx, ctx->alive, alive, size_t(n)))) return rc;
    // Holes in state order (collect, build.go:65-69).
    std::vector<int32_t> holes;
    if (kind)
        for (const uint8_t *q = kind, *end = kind + n;
             (q = static_cast<const uint8_t *>(std::memchr(q, GBH_BLACK_HOLE, size_t(end - q)))) != nullptr; ++q)
            if (!alive || alive[q - kind]) holes.push_back(int32_t(q - kind));
    CK(grow(ctx->holes, ctx->holes_cap, int64_t(holes.size()) + 1));
    if (!holes.empty() && (rc = h2d(ctx, ctx->holes, holes.data(), holes.size() * sizeof(int32_t)))) return rc;
    Launch L = launch_of(ctx);
    int leaf = leaf_of(p);
    double theta = std::min(theta_of(p), 0.9);  // diagTheta, potential.go:12-14
    // FP64 walk: the reference's sums bit for bit; other walks: the mixed walk's potential
    const bool fp64 = p->walk == GBH_WALK_FP64;
    CK(gbh::tree_alloc(ctx->tb, n, leaf, 1));
    ctx->tb.group = 64;
    CK(gbh::tree_build(L, ctx->tb, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind ? ctx->kind : nullptr,
                       alive ? ctx->alive : nullptr, ctx->ax, ctx->ay, ctx->az, theta, leaf, p->dark_matter_off, fp64,
                       false));
    int64_t nparts = (ctx->tb.cap_n + 255) / 256;
    CK(grow(ctx->part, ctx->part_cap, nparts));
    if (!ctx->scalar) CK(gbh::dev_alloc(&ctx->scalar, 256));
    double eps2 = p->softening * p->softening;
    if (fp64) {
        CK(gbh::potential_fp64(L, ctx->tb, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind ? ctx->kind : nullptr,
                               alive ? ctx->alive : nullptr, ctx->holes, int32_t(holes.size()), eps2, c,
                               p->dark_matter_off, !p->monopole_only, ctx->part, ctx->scalar));
    } else {
        CK(grow(ctx->scratch3, ctx->scratch3_cap, 3 * ctx->tb.cap_n));
        CK(gbh::potential_mixed(L, ctx->tb, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind ? ctx->kind : nullptr,
                                alive ? ctx->alive : nullptr, ctx->holes, int32_t(holes.size()), eps2, c,
                                p->dark_matter_off, !p->monopole_only, ctx->scratch3, ctx->part, ctx->scalar));
    }
    if ((rc = d2h(ctx, u, ctx->scalar, sizeof(double)))) return rc;
    return finish(ctx, true);
}

int gbh_direct_accelerations(gbh_ctx *ctx, const gbh_params *p, int64_t n, const double *px, const double *py,
                             const double *pz, const double *mass, const uint8_t *kind, const int64_t *targets,
                             int64_t ntargets, double *ax, double *ay, double *az) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc || (rc = check_params(ctx, p))) return rc;
    if (n < 0 || n > (int64_t(1) << 30)) return fail(ctx, GBH_ERR_ARG, "n out of range");
    if (!targets) ntargets = n;
    if (ntargets < 0) return fail(ctx, GBH_ERR_ARG, "ntargets < 0");
    if (n == 0 || ntargets == 0) return GBH_OK;
    if (!px || !py || !pz || !mass || !ax || !ay || !az) return fail(ctx, GBH_ERR_ARG, "array argument is NULL");
    if (targets)
        for (int64_t q = 0; q < ntargets; ++q)
            if (targets[q] < 0 || targets[q] >= n) return fail(ctx, GBH_ERR_ARG, "target %lld out of range", (long long)q);
    CK(ensure_state(ctx, n));
    ctx->have_state = false;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    size_t b = sizeof(double) * size_t(n);
    if ((rc = h2d(ctx, ctx->px, px, b)) || (rc = h2d(ctx, ctx->py, py, b)) || (rc = h2d(ctx, ctx->pz, pz, b)) ||
        (rc = h2d(ctx, ctx->mass, mass, b)))
        return rc;
    if (kind && (rc = h2d(ctx, ctx->kind, kind, size_t(n)))) return rc;
    CK(grow_targets(ctx, ntargets));
    if (targets && (rc = h2d(ctx, ctx->targets, targets, sizeof(int64_t) * size_t(ntargets)))) return rc;
    double *tx = ctx->tout, *ty = tx + ctx->targets_cap, *tz = ty + ctx->targets_cap;
    Launch L = launch_of(ctx);
    CK(gbh::direct_fp64(L, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind ? ctx->kind : nullptr,
                        p->softening * p->softening, p->dark_matter_off, targets ? ctx->targets : nullptr, ntargets,
                        tx, ty, tz));
    size_t tb = sizeof(double) * size_t(ntargets);
    if ((rc = d2h(ctx, ax, tx, tb)) || (rc = d2h(ctx, ay, ty, tb)) || (rc = d2h(ctx, az, tz, tb))) return rc;
    return finish(ctx, false);
}

int gbh_step_kdk(gbh_ctx *ctx, const gbh_params *p, double dt, int64_t nsteps, int32_t acc_valid, int64_t n,
                 double *px, double *py, double *pz, double *vx, double *vy, double *vz, double *ax, double *ay,
                 double *az, const double *mass, const uint8_t *kind, const uint8_t *alive) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc || (rc = check_params(ctx, p))) return rc;
    if (nsteps < 0) return fail(ctx, GBH_ERR_ARG, "nsteps < 0");
    if (!ax || !ay || !az) return fail(ctx, GBH_ERR_ARG, "acceleration arrays must not be NULL");
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    rc = upload_state(ctx, n, px, py, pz, vx, vy, vz, acc_valid ? ax : nullptr, acc_valid ? ay : nullptr,
                      acc_valid ? az : nullptr, mass, kind, alive);
    if (rc) return rc;
    ctx->last_substeps = 1;
    if (n > 0 && (rc = ctx->state_holes ? run_split_steps(ctx, p, dt, nsteps) : run_steps(ctx, p, dt, nsteps)))
        return rc;
    if (n > 0 && ctx->evused >= 3) {
        // The positions are final once the last force evaluation starts (its first stage event):
        // copy them back on the copy stream while that tree build and walk run.
        size_t b = sizeof(double) * size_t(n);
        CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->evpool[ctx->evused - 3], 0));
        double *dst[3] = {px, py, pz};
        const double *src[3] = {ctx->px, ctx->py, ctx->pz};
        for (int k = 0; k < 3; ++k) {
            CK(cudaMemcpyAsync(dst[k], src[k], b, cudaMemcpyDeviceToHost, ctx->copy_stream));
            ctx->d2h += int64_t(b);
        }
        cudaError_t e = cudaEventRecord(ctx->copy_done, ctx->copy_stream);
        if (e == cudaSuccess) rc = download_state(ctx, nullptr, nullptr, nullptr, vx, vy, vz, ax, ay, az);
        if (e == cudaSuccess && rc == GBH_OK) e = cudaStreamWaitEvent(ctx->stream, ctx->copy_done, 0);
        if (e != cudaSuccess || rc != GBH_OK) {
            cudaStreamSynchronize(ctx->copy_stream);  // no copy into the caller's arrays after return
            return rc != GBH_OK ? rc : fail(ctx, GBH_ERR_CUDA, "position copy: %s", cudaGetErrorString(e));
        }
    } else if ((rc = download_state(ctx, px, py, pz, vx, vy, vz, ax, ay, az))) {
        return rc;
    }
    return finish(ctx, n > 0);
}

int gbh_state_upload(gbh_ctx *ctx, int64_t n, const double *px, const double *py, const double *pz, const double *vx,
                     const double *vy, const double *vz, const double *ax, const double *ay, const double *az,
                     const double *mass, const uint8_t *kind, const uint8_t *alive) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    if ((rc = upload_state(ctx, n, px, py, pz, vx, vy, vz, ax, ay, az, mass, kind, alive))) return rc;
    return finish(ctx, false);
}

int gbh_state_download(gbh_ctx *ctx, double *px, double *py, double *pz, double *vx, double *vy, double *vz, double *ax,
                       double *ay, double *az) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ctx->have_state) return fail(ctx, GBH_ERR_STATE, "no resident state");
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    if ((rc = download_state(ctx, px, py, pz, vx, vy, vz, ax, ay, az))) return rc;
    return finish(ctx, false);
}

int gbh_state_step(gbh_ctx *ctx, const gbh_params *p, double dt, int64_t nsteps) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc || (rc = check_params(ctx, p))) return rc;
    if (!ctx->have_state) return fail(ctx, GBH_ERR_STATE, "no resident state (gbh_state_upload first)");
    if (nsteps < 0) return fail(ctx, GBH_ERR_ARG, "nsteps < 0");
    if (ctx->state_holes && ctx->nsys > 1)
        return fail(ctx, GBH_ERR_UNSUPPORTED, "alive black holes in a forest: the split step couples all systems");
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    ctx->last_substeps = 1;
    if (ctx->n > 0 &&
        (rc = ctx->state_holes ? run_split_steps(ctx, p, dt, nsteps) : run_steps(ctx, p, dt, nsteps)))
        return rc;
    return finish(ctx, ctx->n > 0);
}

int gbh_state_step_block(gbh_ctx *ctx, const gbh_params *p, double dt, double eta, int32_t levels, int64_t nsteps,
                         gbh_blockstats *stats) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc || (rc = check_params(ctx, p))) return rc;
    if (!ctx->have_state) return fail(ctx, GBH_ERR_STATE, "no resident state (gbh_state_upload first)");
    if (nsteps < 0) return fail(ctx, GBH_ERR_ARG, "nsteps < 0");
    if (levels < 1 || levels > 16) return fail(ctx, GBH_ERR_ARG, "levels %d outside [1, 16]", levels);
    if (!(eta > 0)) return fail(ctx, GBH_ERR_ARG, "eta must be > 0");
    if (!(dt > 0)) return fail(ctx, GBH_ERR_ARG, "dt must be > 0");
    if (ctx->state_holes)
        return fail(ctx, GBH_ERR_UNSUPPORTED,
                    "block steps with alive black holes: use gbh_state_step (the hole-aware split step)");
    if (ctx->nsys > 1) return fail(ctx, GBH_ERR_UNSUPPORTED, "block steps of a forest are not supported");
    if (stats) *stats = gbh_blockstats{};
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    if (ctx->n > 0 && (rc = run_block_steps(ctx, p, dt, eta, levels, nsteps, stats))) return rc;
    return finish(ctx, ctx->n > 0);
}

int gbh_state_accelerations(gbh_ctx *ctx, const gbh_params *p) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc || (rc = check_params(ctx, p))) return rc;
    if (!ctx->have_state) return fail(ctx, GBH_ERR_STATE, "no resident state (gbh_state_upload first)");
    if (ctx->n == 0) return GBH_OK;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    rc = forces(ctx, p, ctx->n, ctx->px, ctx->py, ctx->pz, ctx->mass, ctx->state_has_kind ? ctx->kind : nullptr,
                ctx->state_has_alive ? ctx->alive : nullptr, ctx->ax, ctx->ay, ctx->az, theta_of(p), true);
    if (rc) return rc;
    ctx->acc_valid = true;
    return finish(ctx, true);
}

int gbh_state_diagnostics(gbh_ctx *ctx, const gbh_params *p, double c, gbh_diagnostics *out) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc || (rc = check_params(ctx, p))) return rc;
    if (!ctx->have_state) return fail(ctx, GBH_ERR_STATE, "no resident state (gbh_state_upload first)");
    if (!out) return fail(ctx, GBH_ERR_ARG, "out is NULL");
    if (!ctx->have_state) return fail(ctx, GBH_ERR_STATE, "no resident state (gbh_state_upload first)");
    *out = gbh_diagnostics{};
    if (ctx->n == 0) return GBH_OK;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    const int64_t n = ctx->n;
    const uint8_t *kind = ctx->state_has_kind ? ctx->kind : nullptr;
    const uint8_t *alive = ctx->state_has_alive ? ctx->alive : nullptr;
    Launch L = launch_of(ctx);
    CK(grow(ctx->part, ctx->part_cap, std::max<int64_t>((ctx->cap + 255) / 256, int64_t(gbh::diag_parts()) * 11)));
    if (!ctx->scalar) CK(gbh::dev_alloc(&ctx->scalar, 256));
    // potential: the tree at min(theta, 0.9) with the FP64 walk (potential.go:12-42)
    const std::vector<int32_t> &holes = ctx->hole_list;  // alive holes of the state, from its upload
    CK(grow(ctx->holes, ctx->holes_cap, int64_t(holes.size()) + 1));
    if (!holes.empty()) CK(cudaMemcpy(ctx->holes, holes.data(), holes.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    int leaf = leaf_of(p);
    double theta = std::min(theta_of(p), 0.9);
    const bool forest = ctx->nsys > 1;
    // TotalEnergy (diag.go:31-40): the exact pair sum up to exactEnergyLimit bodies, else the tree
    const bool exact = !forest && n <= gbh::kExactEnergyLimit;
    CK(grow(ctx->scratch3, ctx->scratch3_cap, 3 * n));
    double *sa = ctx->scratch3;
    if (exact) {
        CK(gbh::potential_exact_fp64(L, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind, p->softening * p->softening,
                                     c, p->dark_matter_off, sa, ctx->scalar));
    } else {
        // the build zeroes alive holes' accelerations: use the force scratch of the potential path.
        // FP64 walk: the reference's sums bit for bit; other walks: the mixed walk's potential.
        const bool fp64 = p->walk == GBH_WALK_FP64;
        CK(gbh::tree_alloc(ctx->tb, n, leaf, ctx->nsys));
        CK(grow(ctx->scratch3, ctx->scratch3_cap, 3 * ctx->tb.cap_n));
        sa = ctx->scratch3;
        ctx->tb.group = 64;
        CK(gbh::tree_build(L, ctx->tb, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind, alive, sa, sa + n, sa + 2 * n,
                           theta, leaf, p->dark_matter_off, fp64, fp64, forest ? ctx->sys_of : nullptr,
                           forest ? ctx->sys_off : nullptr));
        if (fp64) {
            CK(gbh::potential_fp64(L, ctx->tb, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind, alive, ctx->holes,
                                   int32_t(holes.size()), p->softening * p->softening, c, p->dark_matter_off,
                                   !p->monopole_only, ctx->part, ctx->scalar));
        } else {
            CK(gbh::potential_mixed(L, ctx->tb, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kind, alive, ctx->holes,
                                    int32_t(holes.size()), p->softening * p->softening, c, p->dark_matter_off,
                                    !p->monopole_only, sa, ctx->part, ctx->scalar));
        }
    }
    double u = 0;
    CK(cudaMemcpyAsync(&u, ctx->scalar, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(wait_stream(ctx));
    double sums[11];
    CK(gbh::diagnostics(L, n, ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy, ctx->vz, ctx->mass, kind, c,
                        p->dark_matter_off, ctx->part, ctx->scalar));
    CK(cudaMemcpyAsync(sums, ctx->scalar, sizeof sums, cudaMemcpyDeviceToHost, ctx->stream));
    rc = finish(ctx, !exact);
    if (rc) return rc;
    out->kinetic = sums[0];
    out->potential = u;
    out->total = sums[0] + u;
    out->quality = exact ? 2 : 1;
    for (int k = 0; k < 3; ++k) {
        out->momentum[k] = sums[1 + k];
        out->angular_momentum[k] = sums[4 + k];
        out->center_of_mass[k] = sums[10] != 0 ? sums[7 + k] / sums[10] : 0.0;
    }
    out->mass = sums[10];
    return GBH_OK;
}

int gbh_forest_upload(gbh_ctx *ctx, int32_t nsys, const int64_t *offsets, const double *px, const double *py,
                      const double *pz, const double *vx, const double *vy, const double *vz, const double *ax,
                      const double *ay, const double *az, const double *mass, const uint8_t *kind,
                      const uint8_t *alive) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc) return rc;
    if (nsys < 1 || nsys > 65535) return fail(ctx, GBH_ERR_ARG, "nsys %d outside [1, 65535]", nsys);
    if (!offsets) return fail(ctx, GBH_ERR_ARG, "offsets is NULL");
    if (offsets[0] != 0) return fail(ctx, GBH_ERR_ARG, "offsets[0] must be 0");
    for (int32_t q = 0; q < nsys; ++q)
        if (offsets[q + 1] < offsets[q]) return fail(ctx, GBH_ERR_ARG, "offsets decrease at system %d", q);
    const int64_t n = offsets[nsys];
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    if ((rc = upload_state(ctx, n, px, py, pz, vx, vy, vz, ax, ay, az, mass, kind, alive))) return rc;
    std::vector<uint16_t> sys(static_cast<size_t>(n));
    for (int32_t q = 0; q < nsys; ++q)
        for (int64_t i = offsets[q]; i < offsets[q + 1]; ++i) sys[size_t(i)] = uint16_t(q);
    CK(grow(ctx->sys_of, ctx->sys_of_cap, n + 1));
    CK(grow(ctx->sys_off, ctx->sys_off_cap, int64_t(nsys) + 1));
    if (n > 0) CK(cudaMemcpy(ctx->sys_of, sys.data(), sizeof(uint16_t) * size_t(n), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->sys_off, offsets, sizeof(int64_t) * size_t(nsys + 1), cudaMemcpyHostToDevice));
    ctx->h2d += int64_t(sizeof(uint16_t) * size_t(n) + sizeof(int64_t) * size_t(nsys + 1));
    ctx->nsys = nsys;
    ++ctx->sys_gen;
    return finish(ctx, false);
}

int gbh_forest_layout(gbh_ctx *ctx, int32_t nsys, int64_t *star_range, int64_t *node_range) {
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ctx->tb.info || !ctx->tb.geo) return fail(ctx, GBH_ERR_STATE, "no tree built yet");
    if (nsys != ctx->tb.nsys) return fail(ctx, GBH_ERR_ARG, "the last tree has %d systems", ctx->tb.nsys);
    std::vector<gbh::SysGeo> geo(static_cast<size_t>(nsys));
    CK(cudaMemcpy(geo.data(), ctx->tb.geo, sizeof(gbh::SysGeo) * size_t(nsys), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&ctx->info_host, ctx->tb.info, sizeof(DevInfo), cudaMemcpyDeviceToHost));
    for (int32_t q = 0; q < nsys; ++q) {
        if (star_range) {
            star_range[2 * q] = geo[size_t(q)].star_lo;
            star_range[2 * q + 1] = geo[size_t(q)].star_hi;
        }
        if (node_range) {
            int64_t lo = geo[size_t(q)].root, hi = lo;
            if (lo >= 0) {  // the next non-empty system's root, or the end of the table
                hi = ctx->info_host.nnodes;
                for (int32_t r = q + 1; r < nsys; ++r)
                    if (geo[size_t(r)].root >= 0) {
                        hi = geo[size_t(r)].root;
                        break;
                    }
            } else {
                lo = hi = 0;
            }
            node_range[2 * q] = lo;
            node_range[2 * q + 1] = hi;
        }
    }
    return GBH_OK;
}

int gbh_tree_size(gbh_ctx *ctx, int64_t *nstars, int64_t *nnodes) {
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ctx->tb.info) return fail(ctx, GBH_ERR_STATE, "no tree built yet");
    CK(cudaMemcpy(&ctx->info_host, ctx->tb.info, sizeof(DevInfo), cudaMemcpyDeviceToHost));
    if (nstars) *nstars = ctx->info_host.nstars;
    if (nnodes) *nnodes = ctx->info_host.nnodes;
    return GBH_OK;
}

int gbh_tree_export(gbh_ctx *ctx, uint64_t *keys, int32_t *order, gbh_node *nodes, int64_t node_cap) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ctx->tb.info) return fail(ctx, GBH_ERR_STATE, "no tree built yet");
    CK(cudaMemcpy(&ctx->info_host, ctx->tb.info, sizeof(DevInfo), cudaMemcpyDeviceToHost));
    int64_t ns = ctx->info_host.nstars, nn = ctx->info_host.nnodes;
    if (keys && ns) CK(cudaMemcpy(keys, ctx->tb.keys, sizeof(uint64_t) * size_t(ns), cudaMemcpyDeviceToHost));
    if (order && ns) CK(cudaMemcpy(order, ctx->tb.order, sizeof(int32_t) * size_t(ns), cudaMemcpyDeviceToHost));
    int64_t cnt = std::min(nn, node_cap);
    if (nodes && cnt > 0) {
        if (!ctx->tb.moments_exact) {  // FP32 upsweep: fill the FP64 fields from the walk records
            Launch L = launch_of(ctx);
            CK(gbh::export_fast_moments(L, ctx->tb));
            CK(wait_stream(ctx));
        }
        CK(cudaMemcpy(nodes, ctx->tb.nodes, sizeof(gbh_node) * size_t(cnt), cudaMemcpyDeviceToHost));
    }
    return GBH_OK;
}

int gbh_fwd_save(gbh_ctx *ctx, const gbh_adjoint_params *ap, int64_t n, const double *px, const double *py,
                 const double *pz, const double *vx, const double *vy, const double *vz, const double *mass,
                 double *out_px, double *out_py, double *out_pz, double *out_vx, double *out_vy, double *out_vz) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc) return rc;
    ctx->adj.valid = false;
    if (!ap) return fail(ctx, GBH_ERR_ARG, "adjoint params are NULL");
    if (!(ap->softening > 0)) return fail(ctx, GBH_ERR_ARG, "softening %g must be > 0", ap->softening);
    if (!(std::isfinite(ap->dt))) return fail(ctx, GBH_ERR_ARG, "dt is not finite");
    if (ap->nsteps < 1 || ap->every < 1) return fail(ctx, GBH_ERR_ARG, "nsteps and every must be >= 1");
    if (ap->precision != GBH_ADJ_FP32 && ap->precision != GBH_ADJ_FP64)
        return fail(ctx, GBH_ERR_ARG, "precision %d", ap->precision);
    if (ap->force != GBH_ADJ_DIRECT && ap->force != GBH_ADJ_TREE) return fail(ctx, GBH_ERR_ARG, "force %d", ap->force);
    const bool tree = ap->force == GBH_ADJ_TREE;
    if (tree && ap->precision != GBH_ADJ_FP32) return fail(ctx, GBH_ERR_ARG, "the tree force runs in FP32 only");
    if (tree && !(ap->theta >= 0 && ap->theta <= 1)) return fail(ctx, GBH_ERR_ARG, "theta %g outside [0, 1]", ap->theta);
    if (tree && ap->leaf_size < 0) return fail(ctx, GBH_ERR_ARG, "leaf_size %d < 0", ap->leaf_size);
    if (n < 1 || n > (int64_t(1) << 26)) return fail(ctx, GBH_ERR_ARG, "n = %lld out of range", (long long)n);
    if (!px || !py || !pz || !vx || !vy || !vz || !mass) return fail(ctx, GBH_ERR_ARG, "array argument is NULL");
    gbh::AdjTape &t = ctx->adj;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    CK(gbh::adj_reserve(t, n, ap->nsteps, ap->every, ap->dt, ap->softening, ap->precision == GBH_ADJ_FP32,
                        ctx->num_sms));
    t.tree = tree;
    if (tree) {  // the context's tree buffers, sized for this state
        t.theta = ap->theta == 0 ? 0.9 : ap->theta;  // bh.go:69-74
        t.leaf = ap->leaf_size > 0 ? ap->leaf_size : 24;
        t.tb = &ctx->tb;
        CK(gbh::tree_alloc(ctx->tb, n, t.leaf, 1));
        CK(gbh::adj_tree_reserve(t.tbs, ctx->tb));
    }
    size_t b = sizeof(double) * size_t(n);
    if ((rc = h2d(ctx, t.x, px, b)) || (rc = h2d(ctx, t.x + n, py, b)) || (rc = h2d(ctx, t.x + 2 * n, pz, b)) ||
        (rc = h2d(ctx, t.v, vx, b)) || (rc = h2d(ctx, t.v + n, vy, b)) || (rc = h2d(ctx, t.v + 2 * n, vz, b)) ||
        (rc = h2d(ctx, t.m, mass, b)))
        return rc;
    t.mark = [](void *c) { return stage_event(static_cast<gbh_ctx *>(c)); };
    t.mark_arg = ctx;
    CK(gbh::adj_forward(launch_of(ctx), t));
    double *outs[6] = {out_px, out_py, out_pz, out_vx, out_vy, out_vz};
    for (int k = 0; k < 6; ++k)
        if (outs[k] && (rc = d2h(ctx, outs[k], (k < 3 ? t.x : t.v) + (k % 3) * n, b))) return rc;
    t.valid = false;
    if ((rc = finish(ctx, false))) return rc;
    t.valid = true;
    return GBH_OK;
}

int gbh_bwd(gbh_ctx *ctx, const double *gx, const double *gy, const double *gz, const double *gvx, const double *gvy,
            const double *gvz, double *dx, double *dy, double *dz, double *dvx, double *dvy, double *dvz, double *dm) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc) return rc;
    gbh::AdjTape &t = ctx->adj;
    if (!t.valid) return fail(ctx, GBH_ERR_STATE, "no adjoint tape: call gbh_fwd_save first");
    const int64_t n = t.n;
    size_t b = sizeof(double) * size_t(n);
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    if (t.tree) {  // other calls since the forward may have resized the context's tree buffers
        CK(gbh::tree_alloc(ctx->tb, n, t.leaf, 1));
        CK(gbh::adj_tree_reserve(t.tbs, ctx->tb));
    }
    const double *gin[6] = {gx, gy, gz, gvx, gvy, gvz};
    for (int k = 0; k < 6; ++k) {
        if (gin[k]) {
            if ((rc = h2d(ctx, t.lam + k * n, gin[k], b))) return rc;
        } else {
            CK(cudaMemsetAsync(t.lam + k * n, 0, b, ctx->stream));
        }
    }
    CK(cudaMemsetAsync(t.lam + 6 * n, 0, b, ctx->stream));
    CK(gbh::adj_backward(launch_of(ctx), t));
    double *outs[7] = {dx, dy, dz, dvx, dvy, dvz, dm};
    for (int k = 0; k < 7; ++k)
        if (outs[k] && (rc = d2h(ctx, outs[k], t.lam + k * n, b))) return rc;
    return finish(ctx, false);
}

int gbh_autotune(gbh_ctx *ctx, const gbh_params *base, const double *thetas, int32_t nthetas, const int32_t *leaves,
                 int32_t nleaves, const int32_t *groups, int32_t ngroups, double rms_bound, int32_t sample,
                 int32_t reps, gbh_params *best, gbh_tune_entry *table, int32_t table_cap, int32_t *ntable) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc || (rc = check_params(ctx, base))) return rc;
    if (!best) return fail(ctx, GBH_ERR_ARG, "best is NULL");
    if (!ctx->have_state || ctx->n <= 0) return fail(ctx, GBH_ERR_STATE, "no resident state to tune on");
    static const double kThetas[] = {0.4, 0.5, 0.7};
    static const int32_t kLeaves[] = {4, 8, 16, 32};
    static const int32_t kGroups[] = {64, 32};
    if (!thetas || nthetas <= 0) thetas = kThetas, nthetas = 3;
    if (!leaves || nleaves <= 0) leaves = kLeaves, nleaves = 4;
    if (!groups || ngroups <= 0) groups = kGroups, ngroups = base->walk == GBH_WALK_MIXED ? 2 : 1;
    if (base->walk != GBH_WALK_MIXED) ngroups = 1;  // only the mixed walk has groups
    for (int32_t a = 0; a < nthetas; ++a)
        if (!(thetas[a] > 0 && thetas[a] <= 1)) return fail(ctx, GBH_ERR_ARG, "theta %g outside (0, 1]", thetas[a]);
    for (int32_t a = 0; a < nleaves; ++a)
        if (leaves[a] < 1 || leaves[a] > 1 << 20) return fail(ctx, GBH_ERR_ARG, "leaf size %d", leaves[a]);
    for (int32_t a = 0; a < ngroups; ++a)
        if (groups[a] != 32 && groups[a] != 64) return fail(ctx, GBH_ERR_ARG, "group size %d (32 or 64)", groups[a]);
    if (!(rms_bound > 0)) return fail(ctx, GBH_ERR_ARG, "rms_bound must be > 0");
    if (sample <= 0) sample = 1024;
    if (reps <= 0) reps = 3;
    const int64_t n = ctx->n;
    const bool forest = ctx->nsys > 1;
    // sample targets: evenly spaced alive non-hole bodies (state indices)
    std::vector<uint8_t> kind, alive;
    if (ctx->state_has_kind) {
        kind.resize(size_t(n));
        CK(cudaMemcpy(kind.data(), ctx->kind, size_t(n), cudaMemcpyDeviceToHost));
    }
    if (ctx->state_has_alive) {
        alive.resize(size_t(n));
        CK(cudaMemcpy(alive.data(), ctx->alive, size_t(n), cudaMemcpyDeviceToHost));
    }
    std::vector<int64_t> elig;
    for (int64_t i = 0; i < n; ++i)
        if ((kind.empty() || kind[size_t(i)] != GBH_BLACK_HOLE) && (alive.empty() || alive[size_t(i)]))
            elig.push_back(i);
    if (elig.empty()) return fail(ctx, GBH_ERR_STATE, "no alive stars to tune on");
    const int64_t ns = std::min<int64_t>(sample, int64_t(elig.size()));
    std::vector<int64_t> idx(static_cast<size_t>(ns));
    for (int64_t q = 0; q < ns; ++q) idx[size_t(q)] = elig[size_t(q * int64_t(elig.size()) / ns)];
    // systems: the FP64 direct sum of each target runs over its own system only
    std::vector<int64_t> off{0, n};
    if (forest) {
        off.resize(size_t(ctx->nsys) + 1);
        CK(cudaMemcpy(off.data(), ctx->sys_off, sizeof(int64_t) * off.size(), cudaMemcpyDeviceToHost));
    }
    CK(grow_targets(ctx, 2 * ns));
    Launch L = launch_of(ctx);
    const double eps2 = base->softening * base->softening;
    std::vector<int64_t> rel(static_cast<size_t>(ns));
    std::vector<double> ref(3 * static_cast<size_t>(ns)), got(3 * static_cast<size_t>(ns));
    {
        size_t s = 0, q0 = 0;
        for (size_t q = 0; q < size_t(ns); ++q) {
            while (idx[q] >= off[s + 1]) ++s;
            rel[q] = idx[q] - off[s];
        }
        CK(cudaMemcpyAsync(ctx->targets, rel.data(), sizeof(int64_t) * size_t(ns), cudaMemcpyHostToDevice, ctx->stream));
        double *tx = ctx->tout, *ty = tx + ns, *tz = ty + ns;
        for (s = 0; q0 < size_t(ns); ++s) {
            size_t q1 = q0;
            while (q1 < size_t(ns) && idx[q1] < off[s + 1]) ++q1;
            if (q1 > q0) {
                int64_t o = off[s];
                CK(gbh::direct_fp64(L, off[s + 1] - o, ctx->px + o, ctx->py + o, ctx->pz + o, ctx->mass + o,
                                    ctx->state_has_kind ? ctx->kind + o : nullptr, eps2, base->dark_matter_off,
                                    ctx->targets + q0, int64_t(q1 - q0), tx + q0, ty + q0, tz + q0));
            }
            q0 = q1;
        }
        CK(cudaMemcpyAsync(ref.data(), ctx->tout, sizeof(double) * 3 * size_t(ns), cudaMemcpyDeviceToHost,
                           ctx->stream));
        CK(cudaMemcpyAsync(ctx->targets + ns, idx.data(), sizeof(int64_t) * size_t(ns), cudaMemcpyHostToDevice,
                           ctx->stream));
        CK(wait_stream(ctx));
    }
    const uint8_t *kd = ctx->state_has_kind ? ctx->kind : nullptr, *al = ctx->state_has_alive ? ctx->alive : nullptr;
    int32_t count = 0, best_k = -1, best_any = -1;
    double best_ms = 0, best_err = 0;
    gbh_tune_entry cur_best = {}, any_best = {};
    for (int32_t a = 0; a < nthetas; ++a)
        for (int32_t b = 0; b < nleaves; ++b)
            for (int32_t c = 0; c < ngroups * 2; ++c) {
                // the list walk also sweeps its list depth unless the caller set one
                const bool lists = base->walk == GBH_WALK_MIXED;
                static const int32_t kDepths[2] = {24, 56};
                if ((c & 1) && !(lists && base->list_depth == 0)) continue;
                gbh_params p = *base;
                p.theta = thetas[a];
                p.leaf_size = leaves[b];
                p.group_size = groups[c / 2];
                p.list_depth = lists ? (base->list_depth ? base->list_depth : kDepths[c & 1]) : 0;
                gbh_tune_entry e = {};
                e.theta = p.theta;
                e.leaf_size = p.leaf_size;
                e.group_size = base->walk == GBH_WALK_MIXED ? (p.group_size == 32 ? 32 : 64) : 0;
                e.list_depth = p.list_depth;
                std::vector<double> tot, bld, wlk;
                for (int32_t r = -1; r < reps; ++r) {  // r = -1: untimed warm-up (allocation)
                    ctx->evused = 0;
                    rc = forces(ctx, &p, n, ctx->px, ctx->py, ctx->pz, ctx->mass, kd, al, ctx->ax, ctx->ay, ctx->az,
                                theta_of(&p), forest);
                    if (rc) return rc;
                    CK(wait_stream(ctx));
                    if (r < 0) continue;
                    float b0 = 0, w0 = 0;
                    CK(cudaEventElapsedTime(&b0, ctx->evpool[0], ctx->evpool[1]));
                    CK(cudaEventElapsedTime(&w0, ctx->evpool[1], ctx->evpool[2]));
                    bld.push_back(b0);
                    wlk.push_back(w0);
                    tot.push_back(double(b0) + double(w0));
                }
                auto median = [](std::vector<double> v) {
                    std::sort(v.begin(), v.end());
                    return v[v.size() / 2];
                };
                e.ms = median(tot);
                e.build_ms = median(bld);
                e.walk_ms = median(wlk);
                k_gather3<<<unsigned((ns + 255) / 256), 256, 0, ctx->stream>>>(ns, ctx->targets + ns, ctx->ax, ctx->ay,
                                                                              ctx->az, ctx->tout);
                ++ctx->launches;
                CK(cudaGetLastError());
                CK(cudaMemcpyAsync(got.data(), ctx->tout, sizeof(double) * 3 * size_t(ns), cudaMemcpyDeviceToHost,
                                   ctx->stream));
                CK(wait_stream(ctx));
                std::vector<double> rerr;
                for (int64_t q = 0; q < ns; ++q) {
                    double rx = ref[size_t(q)], ry = ref[size_t(ns + q)], rz = ref[size_t(2 * ns + q)];
                    double dx = got[size_t(q)] - rx, dy = got[size_t(ns + q)] - ry, dz = got[size_t(2 * ns + q)] - rz;
                    double nr = std::sqrt(rx * rx + ry * ry + rz * rz);
                    if (nr > 0) rerr.push_back(std::sqrt(dx * dx + dy * dy + dz * dz) / nr);
                }
                double s2 = 0;
                for (double x : rerr) s2 += x * x;
                e.rms_err = rerr.empty() ? 0 : std::sqrt(s2 / double(rerr.size()));
                std::sort(rerr.begin(), rerr.end());
                e.p99_err = rerr.empty() ? 0 : rerr[std::min(rerr.size() - 1, size_t(0.99 * double(rerr.size())))];
                e.meets = e.rms_err <= rms_bound;
                if (e.meets && (best_k < 0 || e.ms < best_ms)) best_k = count, best_ms = e.ms, cur_best = e;
                if (best_any < 0 || e.rms_err < best_err) best_any = count, best_err = e.rms_err, any_best = e;
                if (table && count < table_cap) table[count] = e;
                ++count;
            }
    ctx->acc_valid = false;  // the accelerations are those of the last candidate
    const gbh_tune_entry &w = best_k >= 0 ? cur_best : any_best;
    *best = *base;
    best->theta = w.theta;
    best->leaf_size = w.leaf_size;
    best->group_size = w.group_size;
    best->list_depth = w.list_depth;
    if (ntable) *ntable = count;
    ctx->evused = 0;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    rc = finish(ctx, false);
    if (rc) return rc;
    return best_k >= 0 ? GBH_OK : fail(ctx, GBH_ERR_LIMIT, "no candidate meets rms %g (best %g)", rms_bound, best_err);
}

int gbh_last_timings(gbh_ctx *ctx, gbh_timings *t) {
    if (!ctx || !t) return GBH_ERR_ARG;
    *t = ctx->last;
    return GBH_OK;
}

int gbh_probe_fp32_peak(gbh_ctx *ctx, double ms, double *tflops) {
    gbh::NvtxRange nvtx_range_(__func__);
    int rc = begin(ctx);
    if (rc) return rc;
    if (!tflops) return fail(ctx, GBH_ERR_ARG, "tflops is NULL");
    if (!ctx->probe) CK(gbh::dev_alloc(&ctx->probe, sizeof(float) * 65536));
    Launch L = launch_of(ctx);
    int blocks = ctx->num_sms * 8;  // 8 x 256 threads = 64 warps per SM
    int iters = 64;
    // Calibrate the iteration count so one launch lasts about ms.
    for (int round = 0; round < 8; ++round) {
        CK(cudaEventRecord(ctx->ev[0], ctx->stream));
        CK(gbh::fp32_fma_probe(L, blocks, iters, ctx->probe));
        CK(cudaEventRecord(ctx->ev[1], ctx->stream));
        CK(cudaEventSynchronize(ctx->ev[1]));
        float t = 0;
        CK(cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]));
        if (t >= ms * 0.5 || iters > (1 << 24)) {
            double flops = 2.0 * 8 * 16 * double(iters) * double(blocks) * 256;
            // best of 3 at this size
            float best = t;
            for (int r = 0; r < 3; ++r) {
                CK(cudaEventRecord(ctx->ev[0], ctx->stream));
                CK(gbh::fp32_fma_probe(L, blocks, iters, ctx->probe));
                CK(cudaEventRecord(ctx->ev[1], ctx->stream));
                CK(cudaEventSynchronize(ctx->ev[1]));
                CK(cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]));
                best = std::min(best, t);
            }
            *tflops = flops / (double(best) * 1e-3) / 1e12;
            return GBH_OK;
        }
        double scale = t > 0 ? ms / t : 8.0;
        iters = int(std::min<double>(double(iters) * std::min(scale, 16.0), double(1 << 25)));
    }
    return fail(ctx, GBH_ERR_CUDA, "probe did not converge");
}

}  // extern "C"
