/*
 * gbh.h — C-ABI of the GB300 Barnes-Hut gravity step (libgbh.so).
 *
 * This is the drop-in boundary for gravitas' force and step path. The
 * reference binds its force solver through the Go interface
 *     type Solver interface { Accelerations(s *State, p Params) }
 * (internal/sim/sim.go:100-105), implemented by bh.Solver
 * (internal/sim/bh/bh.go:28-102), and reaches native code through cgo static C
 * functions (internal/sim/bh/gpu_darwin.go:18-62: gpu_init / gpu_buffer /
 * gpu_walk, synchronous, 0-or-error-code returns with a message buffer). The
 * entry points below replace those; each cites the reference interface it
 * stands in for. Plain pointers and sizes only; all host arrays are owned by
 * the caller, all device memory by the context (grow-only, no allocation per
 * call once sizes are stable).
 *
 * Threading: a context may be used from any OS thread (it makes its device
 * current on every entry, as a cgo caller can migrate between threads), but
 * by one thread at a time. Every call is synchronous: it returns after the
 * device work it issued has finished, like gpu_walk's waitUntilCompleted.
 *
 * Errors: every function returns GBH_OK (0) or a GBH_ERR_* code; the message
 * is available from gbh_last_error(). Nothing aborts the process.
 */
#ifndef GBH_H
#define GBH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBH_ABI_VERSION 1

enum {
    GBH_OK = 0,
    GBH_ERR_ARG = 1,         /* invalid argument (null pointer, negative size, bad enum), or an
                                alive star with a non-finite position or mass: found on the device
                                by the tree build's bounding-box reduction, before keys are formed
                                (the call's outputs are then undefined) */
    GBH_ERR_CUDA = 2,        /* a CUDA runtime call failed (message has the CUDA error) */
    GBH_ERR_NOMEM = 3,       /* device allocation failed (test hook: with GBH_FAULT_ALLOC=k in the
                                environment when a context is created, the allocation after k
                                successful ones fails once, without touching the device) */
    GBH_ERR_LIMIT = 4,       /* a device-side walk exceeded its step bound (a corrupt tree); the
                                message names the kernel (test hook: with GBH_FAULT_LINK set when a
                                context is created, its next tree gets a cycle in its skip links) */
    GBH_ERR_STATE = 5,       /* no resident state, or sizes do not match it */
    GBH_ERR_UNSUPPORTED = 6  /* input outside this path (e.g. alive black holes in a step) */
};

/* Body kinds, internal/sim/state.go:12-21 (sim.Kind). */
enum { GBH_STAR = 0, GBH_BLACK_HOLE = 1, GBH_DARK_MATTER = 2, GBH_GAS = 3 };

/* Tree walk variants. */
enum {
    /* Warp-cooperative FP32 walk with compensated per-star accumulation and
       separations formed from hi + lo splits of the FP64 positions; every star
       sees each accepted node exactly where the reference walk accepts it, or
       deeper. Two kernels: the list walk, one warp per 32 or 64
       Morton-consecutive stars (one or two a lane; see group_size) that builds
       the group's interaction lists with node-parallel opening tests and
       evaluates them from shared memory two entries at a time in packed FP32x2
       arithmetic, its split mode sharing a group among several warps for small
       systems; and the paired walk (GBH_CFG_PAIRED), one warp per 64 stars
       walking the skip links in lockstep. The default. */
    GBH_WALK_MIXED = 0,
    /* One thread per star, all FP32, uncompensated: the CUDA twin of the Metal
       kernel internal/sim/bh/gpu_darwin.go:76-118. */
    GBH_WALK_PLAIN = 1,
    /* One thread per star in FP64 with the reference's operation order: bit
       identical to bh.Solver.walk (internal/sim/bh/bh.go:106-155). */
    GBH_WALK_FP64 = 2
};

/* Solver knobs: bh.Solver{Theta, MonopoleOnly} (bh.go:29-38) and the
   sim.Params fields the force path reads (sim.go:9-23). */
typedef struct {
    double theta;            /* opening angle; 0 means 0.9 (bh.go:14-16, 69-74) */
    double softening;        /* Plummer softening length eps (Params.Softening) */
    int32_t leaf_size;       /* max stars per leaf; 0 means 24 (bh.go:17-19) */
    int32_t monopole_only;   /* drop quadrupoles of accepted nodes (bh.go:34-35) */
    int32_t dark_matter_off; /* dark matter pulls nothing (Params.DarkMatterOff, sim.go:92-98) */
    int32_t walk;            /* GBH_WALK_* */
    int32_t group_size;      /* GBH_WALK_MIXED: 32 the list walk with one star a lane; 64 with two
                                (the paired walk with GBH_CFG_PAIRED); 0: 64 for a forest and for
                                a single system of at least 524,288 stars, else 32 */
    int32_t list_depth;      /* list walk: node-list entries evaluated per pass, 2 to 56 (0 means 56;
                                source lists take twice as many, up to 160) */
    double c;                /* speed of light of the steps (Params.C): 0 Newtonian; > 0 drifts by
                                u / gamma (sim.go:315-343) and uses Paczynski-Wiita star-hole
                                pairs in the hole-aware step (pair.go:26-35) */
} gbh_params;

enum {
    /* Steps launch their kernels one by one instead of replaying a captured CUDA graph. */
    GBH_CFG_NO_GRAPHS = 1,
    /* Host waits for the GPU sleep on a blocking-sync event instead of spinning, so a caller
       thread blocked in a call (a goroutine running Accelerations while Hydro.Forces runs on
       the other cores, gas.go:20-25) leaves its core free. */
    GBH_CFG_BLOCKING_SYNC = 2,
    /* The mixed walk launches its groups in index order instead of longest first (the order
       the previous walk's group costs give); results are identical either way. */
    GBH_CFG_NO_LPT = 4,
    /* The mixed walk of a single system never splits a group's walk over several warps. With few
       groups (up to 21 per SM: below about 100,000 stars in 32-star groups, 200,000 in 64-star
       groups on a GB300, or as few stars in a block-step event's list) each group's walk is
       otherwise shared by 2 to 32 warps (the split mode of the list walk, or of the paired walk),
       each adding the interactions of its own range of source stars, and the parts are summed
       in order: the same interactions, a different order of summation. */
    GBH_CFG_NO_SPLIT = 8,
    /* 64-star groups of the mixed walk take the paired walk (split or not) instead of the list
       walk. */
    GBH_CFG_PAIRED = 16
};

typedef struct {
    int32_t device;          /* CUDA device ordinal */
    int32_t flags;           /* GBH_CFG_* bits */
    int32_t reserved[6];     /* zero */
} gbh_config;

/* One tree node, field for field internal/sim/bh/bh.go:59-67 (104 bytes). */
typedef struct {
    double x, y, z, m;
    double qxx, qyy, qzz, qxy, qxz, qyz;
    double crit2;
    int32_t first, next, lo, hi;
} gbh_node;

/* Device times of the last call, from CUDA events on the context's stream
   (LastGPUSeconds, gpu_darwin.go:155, split by stage). */
typedef struct {
    double build_ms;   /* collect, keys, sort, node ranges, moments */
    double walk_ms;    /* tree walk */
    double step_ms;    /* kicks and drift */
    double total_ms;   /* everything the call issued, copies included */
    int64_t nstars;    /* stars in the last tree */
    int64_t nnodes;    /* nodes in the last tree */
    int64_t launches;  /* kernels launched by the last call */
    int64_t h2d_bytes; /* host-to-device bytes copied by the last call */
    int64_t d2h_bytes; /* device-to-host bytes copied by the last call */
    int64_t substeps;  /* hole substeps of the last step (Simulation.Substeps, split.go:174); 1 without holes */
} gbh_timings;

typedef struct gbh_ctx gbh_ctx;

/* Creates a context on cfg->device (NULL: device 0). Replaces gpu_init /
   GPUAvailable (gpu_darwin.go:18-29, 132-142): returns a code and writes a
   message to err on failure. */
int gbh_create(const gbh_config *cfg, gbh_ctx **out, char *err, int errlen);
/* Frees the context and all its device memory. NULL is a no-op. */
void gbh_destroy(gbh_ctx *ctx);
/* Message of the last failed call on ctx ("" after a success). */
const char *gbh_last_error(const gbh_ctx *ctx);
/* Device name (GPUName, gpu_darwin.go:145-152). */
int gbh_device_name(gbh_ctx *ctx, char *out, int len);

/*
 * bh.Solver.Accelerations (bh.go:76-102) on host arrays of one sim.State
 * (state.go:33-52): fills ax/ay/az for every alive non-hole body from the
 * star–star forces, sets alive black holes to 0 and leaves dead bodies'
 * entries untouched. kind and alive may be NULL (all stars, all alive).
 */
int gbh_accelerations(gbh_ctx *ctx, const gbh_params *p, int64_t n, const double *px,
                      const double *py, const double *pz, const double *mass,
                      const uint8_t *kind, const uint8_t *alive, double *ax, double *ay,
                      double *az);

/*
 * bh.Solver.PotentialEnergy (potential.go:12-42): U from an FP64 tree walk
 * at min(theta, 0.9), with star–hole and hole–hole pairs in the pair model of
 * internal/sim/pair.go at speed of light c (0: Newtonian).
 */
int gbh_potential_energy(gbh_ctx *ctx, const gbh_params *p, int64_t n, const double *px,
                         const double *py, const double *pz, const double *mass,
                         const uint8_t *kind, const uint8_t *alive, double c, double *u);

/*
 * direct.Solver.Accelerations (internal/sim/direct/direct.go:18-48) in FP64 on
 * the GPU, for the ntargets state indices in targets (all bodies when targets
 * is NULL; then ntargets is ignored and rows follow state order). Same
 * operation order as the reference, so results are bit identical to it.
 */
int gbh_direct_accelerations(gbh_ctx *ctx, const gbh_params *p, int64_t n, const double *px,
                             const double *py, const double *pz, const double *mass,
                             const uint8_t *kind, const int64_t *targets, int64_t ntargets,
                             double *ax, double *ay, double *az);

/*
 * sim.Simulation.Step (sim.go:248-288) repeated nsteps times, without gas hydro, with
 * the speed of light p->c (0: Newtonian). Without alive black holes: kick(dt/2),
 * drift(dt) (sim.go:327-343: x += dt v, or dt u / gamma for c > 0),
 * Solver.Accelerations, kick(dt/2); each step replays one CUDA graph (captured on
 * first use for the sizes and parameters given, re-captured when they change) unless
 * the context was created with GBH_CFG_NO_GRAPHS; results are identical either way.
 * With alive black holes: the hole-aware split step (split.go:162-200, stepSplit):
 * forces of pairs with a hole summed directly with the pair model (pair.go:14-47:
 * Newtonian for c = 0, Paczynski-Wiita star-hole forces for c > 0),
 * stars whose timescale at a hole is below 20 dt and the holes advanced in 2^k
 * substeps (classify, split.go:39-85; k of the last step in gbh_timings.substeps),
 * star-star forces from the tree once per step; no graph (the substep count is read
 * back every step). If acc_valid is 0 the forces are computed first (initForces,
 * gas.go:14-17). Arrays are read and written in place; the state stays on the device
 * between the steps.
 */
int gbh_step_kdk(gbh_ctx *ctx, const gbh_params *p, double dt, int64_t nsteps, int32_t acc_valid,
                 int64_t n, double *px, double *py, double *pz, double *vx, double *vy,
                 double *vz, double *ax, double *ay, double *az, const double *mass,
                 const uint8_t *kind, const uint8_t *alive);

/* ---- Resident state: the same step with the state kept in HBM between calls. ---- */

/* Copies a state to the device (acc may be NULL: forces are then computed before the
   first step). */
int gbh_state_upload(gbh_ctx *ctx, int64_t n, const double *px, const double *py,
                     const double *pz, const double *vx, const double *vy, const double *vz,
                     const double *ax, const double *ay, const double *az, const double *mass,
                     const uint8_t *kind, const uint8_t *alive);
/* Copies the resident state back (any pointer may be NULL). */
int gbh_state_download(gbh_ctx *ctx, double *px, double *py, double *pz, double *vx, double *vy,
                       double *vz, double *ax, double *ay, double *az);
/* nsteps KDK steps on the resident state (as gbh_step_kdk, no copies). A forest with alive
   black holes returns GBH_ERR_UNSUPPORTED (the split step would couple its systems). */
int gbh_state_step(gbh_ctx *ctx, const gbh_params *p, double dt, int64_t nsteps);
/* Statistics of block steps. */
typedef struct {
    int64_t substeps;          /* events: tree builds and walks of the active stars */
    int64_t evaluations;       /* stars walked, summed over the events */
    int32_t min_substep_ticks; /* shortest interval between events, in ticks of dt / 2^(levels-1) */
    int32_t reserved;
} gbh_blockstats;

/*
 * nsteps global steps of length dt with power-of-two block time steps on the resident state.
 * The reference steps gravity with one global dt; this follows its gas block steps
 * (internal/sim/blockstep.go:22-90): a body's rung is the smallest r with dt / 2^r <= dt_i
 * (rungFor, blockstep.go:38-45), capped at levels - 1, with dt_i = eta * sqrt(softening / |a_i|),
 * and a step may start only at a multiple of its length (blockstep.go:84-86). Kick-drift-kick
 * per body: opening half kick when its step starts, all bodies drift together from event to
 * event, the tree of all stars is rebuilt at each event and only the bodies whose step ends
 * are walked, kicked and given a new rung. levels = 1 is exactly gbh_state_step. stats may be
 * NULL.
 */
int gbh_state_step_block(gbh_ctx *ctx, const gbh_params *p, double dt, double eta, int32_t levels,
                         int64_t nsteps, gbh_blockstats *stats);
/* Accelerations of the resident state (as gbh_accelerations, no copies). */
int gbh_state_accelerations(gbh_ctx *ctx, const gbh_params *p);

/* Conserved quantities of the resident state (internal/sim/diag.go:31-135), FP64 on the
   GPU. */
typedef struct {
    double kinetic;             /* sourceKinetic: sum of m u^2 / (gamma + 1) over bodies that gravitate (diag.go:66-76) */
    double potential;           /* exact pair sum for up to 30,000 bodies (PotentialEnergyParallel,
                                   diag.go:42-64), else the tree potential at min(theta, 0.9)
                                   (potential.go:12-42); forests always use the tree */
    double total;               /* kinetic + potential (TotalEnergy without gas, diag.go:31-40) */
    double momentum[3];         /* Momentum, all bodies (diag.go:102-110) */
    double angular_momentum[3]; /* AngularMomentum about the origin (diag.go:112-120) */
    double center_of_mass[3];   /* CenterOfMass (diag.go:122-135) */
    double mass;                /* its total mass */
    int32_t quality;            /* EnergyQuality (diag.go:21-27): 2 exact, 1 tree estimate */
    int32_t reserved;
} gbh_diagnostics;

/* Diagnostics of the resident state; c is the speed of light of the pair model (0: Newtonian). */
int gbh_state_diagnostics(gbh_ctx *ctx, const gbh_params *p, double c, gbh_diagnostics *out);

/* ---- Batched forest: many independent systems in one resident state. ---- */

/*
 * Uploads nsys independent systems (at most 65,535) as one resident state: the bodies of
 * system s are [offsets[s], offsets[s+1]) (offsets[0] = 0, n = offsets[nsys]); the other
 * arrays are as in gbh_state_upload. Each system gets its own tree, exactly the tree
 * bh.Solver builds for that system alone (its own root cube, keys, node layout); one build
 * and one walk launch serve all systems. gbh_state_step, gbh_state_accelerations,
 * gbh_state_diagnostics and gbh_state_download then act on the forest; gbh_state_upload
 * returns to a single system. Block steps are not available for forests.
 */
int gbh_forest_upload(gbh_ctx *ctx, int32_t nsys, const int64_t *offsets, const double *px,
                      const double *py, const double *pz, const double *vx, const double *vy,
                      const double *vz, const double *ax, const double *ay, const double *az,
                      const double *mass, const uint8_t *kind, const uint8_t *alive);
/* Layout of the last forest tree: for system s, star_range[2s..2s+1] is its sorted star range
   in gbh_tree_export's keys/order and node_range[2s..2s+1] its node range in the node table
   (links inside are table indices; a system's root is node_range[2s]). Either may be NULL. */
int gbh_forest_layout(gbh_ctx *ctx, int32_t nsys, int64_t *star_range, int64_t *node_range);

/* ---- Adjoint pair: gradient of a loss on the final phase-space coordinates. ---- */

/*
 * No counterpart in the reference (it has no differentiable path). Differentiates N KDK steps
 * (the step of gbh_step_kdk, sim.go:302-343) with the softened O(N^2) direct-sum force
 * (direct.go:27-47), every body a star: the force whose gradient finite differences can check,
 * because the tree force jumps where a node's opening test or a star's cell changes.
 */
enum { GBH_ADJ_FP32 = 0, GBH_ADJ_FP64 = 1 };
enum { GBH_ADJ_DIRECT = 0, GBH_ADJ_TREE = 1 };
typedef struct {
    double dt;         /* step length */
    double softening;  /* Plummer epsilon; must be > 0 */
    int64_t nsteps;    /* >= 1 */
    int64_t every;     /* checkpoint interval K >= 1: (x, v, a) saved every K steps */
    int32_t precision; /* GBH_ADJ_FP64: pair sums in the FP64 reference order (j ascending);
                          GBH_ADJ_FP32: FP32 pairs, double-float separations, compensated sums */
    int32_t force;     /* GBH_ADJ_DIRECT: the softened direct sum (direct.go:18-48), every body a
                          source; GBH_ADJ_TREE (GBH_ADJ_FP32 only): the Barnes-Hut force of the
                          mixed walk (quadrupoles, 32-star groups of the list walk, FP32 moments),
                          differentiated with each step's interaction lists and tree topology
                          frozen (the lists the forward builds at the same positions) */
    int32_t leaf_size; /* GBH_ADJ_TREE: max stars per leaf; 0 means 24 */
    int32_t reserved;
    double theta;      /* GBH_ADJ_TREE: opening angle; 0 means 0.9 */
} gbh_adjoint_params;

/* Forward half: runs the steps from (x0, v0) with masses m, keeping checkpoints on the
   device, and returns the final positions and velocities (any out pointer may be NULL).
   The tape stays in the context until the next gbh_fwd_save or gbh_destroy. */
int gbh_fwd_save(gbh_ctx *ctx, const gbh_adjoint_params *ap, int64_t n, const double *px,
                 const double *py, const double *pz, const double *vx, const double *vy,
                 const double *vz, const double *mass, double *out_px, double *out_py,
                 double *out_pz, double *out_vx, double *out_vy, double *out_vz);
/* Backward half: given dL/dx_T and dL/dv_T (NULL arrays are zero), returns dL/dx_0, dL/dv_0
   and dL/dm (any out pointer may be NULL) by replaying each checkpoint segment. It may be
   called again on the same tape with another loss. GBH_ERR_STATE without a tape. */
int gbh_bwd(gbh_ctx *ctx, const double *gx, const double *gy, const double *gz, const double *gvx,
            const double *gvy, const double *gvz, double *dx, double *dy, double *dz, double *dvx,
            double *dvy, double *dvz, double *dm);

/* ---- Autotuner. ---- */

/* One candidate of gbh_autotune. */
typedef struct {
    double theta;
    int32_t leaf_size;
    int32_t group_size; /* 32 or 64 for GBH_WALK_MIXED, 0 for the other walks */
    double ms;          /* median device time of one force evaluation (build + walk) */
    double build_ms;    /* its tree build */
    double walk_ms;     /* its walk */
    double rms_err;     /* RMS of the per-body relative force error on the sample */
    double p99_err;     /* 99th percentile of the same */
    int32_t meets;      /* rms_err <= rms_bound */
    int32_t list_depth; /* mixed walk: its list walk's node-list depth; 0 for the other walks */
} gbh_tune_entry;

/*
 * No counterpart in the reference (its internal/perf/calibrate.go only picks CPU or GPU).
 * Sweeps theta x leaf size x group size on the resident state (gbh_state_upload or
 * gbh_forest_upload) with the other fields of *base, and writes to *best the candidate with
 * the shortest median force evaluation (reps timed runs, CUDA events) among those whose RMS
 * relative force error, on `sample` evenly spaced alive stars against the FP64 direct sum
 * over each star's own system, is at most rms_bound. NULL or empty lists take the defaults
 * theta {0.4, 0.5, 0.7}, leaf {4, 8, 16, 32}, group {64, 32}, and for the mixed walk the list
 * depths {24, 56} unless base->list_depth is set; sample <= 0 means 1024 and
 * reps <= 0 means 3. Every candidate is written to table (up to table_cap) and counted in
 * *ntable. If none meets the bound, *best is the most accurate one and the call returns
 * GBH_ERR_LIMIT. The resident accelerations are left stale (the next step recomputes them).
 */
int gbh_autotune(gbh_ctx *ctx, const gbh_params *base, const double *thetas, int32_t nthetas,
                 const int32_t *leaves, int32_t nleaves, const int32_t *groups, int32_t ngroups,
                 double rms_bound, int32_t sample, int32_t reps, gbh_params *best,
                 gbh_tune_entry *table, int32_t table_cap, int32_t *ntable);

/* ---- Inspection of the last tree (b.nodes / b.order / b.keys in bh.Solver). ---- */

/* Stars and nodes of the last built tree. */
int gbh_tree_size(gbh_ctx *ctx, int64_t *nstars, int64_t *nnodes);
/* Copies the last tree: Morton keys and state indices in sorted order (nstars each)
   and the node table in the reference's serial index layout (up to node_cap nodes).
   Any pointer may be NULL. Keys, order, ranges and links are always the reference's;
   the moments are the reference's FP64 values, bit for bit, after a GBH_WALK_FP64 call,
   and FP32-accurate values after a call with an FP32 walk. */
int gbh_tree_export(gbh_ctx *ctx, uint64_t *keys, int32_t *order, gbh_node *nodes,
                    int64_t node_cap);
/* Device times and counters of the last call. */
int gbh_last_timings(gbh_ctx *ctx, gbh_timings *t);

/* ---- Diagnostics. ---- */

/* Measures this device's FP32 FMA throughput (TFLOP/s, 2 flops per FMA) with a
   register-resident FMA loop of about ms milliseconds; the roofline denominator
   of the walk. */
int gbh_probe_fp32_peak(gbh_ctx *ctx, double ms, double *tflops);

/* ---- Without device allocation. ---- */

/*
 * No counterpart in the reference. For callers that must not call cudaMalloc: code whose
 * device memory belongs to another framework's allocator that has already reserved most of
 * the GPU, code that cannot take the device-wide synchronisation cudaMalloc/cudaFree may
 * imply while other streams run, and loops that must never allocate after start-up.
 *
 * Sorted Morton keys and state indices of the alive non-hole bodies, exactly the keys and
 * order gbh_tree_export returns after gbh_accelerations on the same arrays (collect, keys
 * and the stable radix sort of the tree build). All pointers except nstars, err and stream
 * are device pointers owned by the caller: px/py/pz hold n doubles, kind/alive n bytes (each
 * may be NULL: all stars, all alive), keys and order room for n entries; *nstars (host)
 * receives the number of sorted bodies. stream is a cudaStream_t (NULL: the legacy default
 * stream); the call returns after the work on it has finished.
 *
 * It allocates nothing: its temporaries live in one static device array of 4.5 MiB that
 * every GPU which loads the library holds until the process exits, enough for at most
 * 262,144 bodies; larger n returns GBH_ERR_ARG. The first call on a device looks up that
 * array's device address, so make it before any stream capture. The address is kept for the
 * life of the process: after a cudaDeviceReset of that device, do not call this entry point on
 * it again. All calls share the array: calls that overlap on the GPU (for instance on two
 * streams of one device) race and must be serialised by the caller. Every call waits for its
 * stream to finish before returning (it reads the number of sorted bodies back to the host), so
 * it cannot be called while that stream is being captured into a CUDA graph.
 * An alive star with a non-finite position gives GBH_ERR_ARG. Errors are returned as a code
 * with a message in err.
 */
int gbh_morton_order_noalloc(int32_t device, void *stream, int64_t n, const double *px,
                             const double *py, const double *pz, const uint8_t *kind,
                             const uint8_t *alive, uint64_t *keys, int32_t *order,
                             int64_t *nstars, char *err, int errlen);

#ifdef __cplusplus
}
#endif
#endif
