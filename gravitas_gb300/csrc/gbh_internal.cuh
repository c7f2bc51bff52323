// Internal declarations shared by the CUDA translation units of libgbh.
//
// Layout in HBM (one context, one tree at a time):
//   state, state order (SoA FP64): px py pz vx vy vz ax ay az mass, kind/alive u8
//   sorted stars: keys u64, order i32, sx sy sz sm FP64, st_hi/st_lo float4
//   nodes, reference serial index layout: gbh_node (104 B) + walk records
//     PNode (64 B, FP32, the Metal GNode) and MNode (64 B, hi/lo FP32) + int2 ranges
#pragma once

#include <cuda_runtime.h>

#include <vector>
#include <stdint.h>

#include "../../include/gbh.h"

namespace gbh {

constexpr int kMortonBits = 21;           // morton.go:4
constexpr int kMaxLevel = kMortonBits;    // buildNode splits only below level 21 (build.go:136)
constexpr int kNoCell = 22;               // "starts no cell": duplicate of the previous key

// DevInfo.err_where of a build whose alive stars include a non-finite position or mass (the
// caller gets GBH_ERR_ARG); every other value names the kernel whose bound or check failed
// (GBH_ERR_LIMIT).
constexpr int kErrNonFinite = 20;
// A one-sweep sort pass or a single-pass scan whose look-back wait ran past its bound.
constexpr int kErrSortWait = 30;
constexpr int kErrScanWait = 31;

// Per-build scalars kept on the device, so a step needs no host round trip.
struct DevInfo {
    double minx, miny, minz;  // bbox min of the stars (build.go:12)
    double side;              // root cube side (build.go:19-20)
    double scale;             // 2^21 / side (build.go:21)
    double theta;             // opening angle used for crit2
    int64_t nstars;           // alive non-hole bodies
    int64_t nnodes;           // nodes of the tree
    int32_t err;              // device-side limit hit (walk step bound, stack bound)
    int32_t err_where;        // which kernel set err
    uint32_t work;            // work counter of persistent kernels
    uint32_t nleaves;         // leaves appended to the leaf list
    uint32_t ntargets;        // entries of the target list (walks restricted to active stars)
    uint32_t ngroups;         // mixed-walk groups of a forest
    int32_t next_tick;        // block steps: the earliest step end over all bodies
    uint32_t next_count;      // block steps: the bodies whose step ends at next_tick
    // FP32 views for the FP32 upsweep: min corner and side as hi + lo pairs, and the
    // opening base 2 * half_L / theta per level L
    float min_hi[3], min_lo[3];
    float side_hi, side_lo;
    float crit_base[kMaxLevel + 1];
};

// Geometry and layout of one system of a forest (a single state is a forest of one system):
// its root cube, FP32 views of it, the opening bases per level, its sorted star range, its
// root node and its first mixed-walk group.
struct SysGeo {
    double minx, miny, minz, side, scale;
    float min_hi[3], min_lo[3];
    float side_hi, side_lo;
    float crit_base[kMaxLevel + 1];
    long long kmin[3], kmax[3];  // ordered keys of the bbox (accumulated by atomics)
    int32_t star_lo, star_hi;    // sorted range of its stars
    int32_t root;                // index of its root node; its nodes follow in its own serial layout
    int32_t group_lo, ngroups;   // its 64-star mixed-walk groups
    int32_t pad;
};

// The Metal kernel's GNode (gpu_darwin.go:79,121-124): com (x,y,z,m), q1 (qxx,qyy,qzz,qxy),
// q2 (qxz,qyz,crit2,0), links (first,next,lo,hi).
struct __align__(16) PNode {
    float4 com, q1, q2;
    int4 links;
};

// Mixed-walk node: a = (com_hi.xyz, crit2), b = (com_lo.xyz, m), c = (qxx,qyy,qzz,qxy),
// d = (qxz, qyz, first as bits, next as bits). com = com_hi + com_lo (FP64 split in two FP32).
struct __align__(16) MNode {
    float4 a, b, c, d;
};

// List-walk node: a = (com_hi.xyz, crit), b = (com_lo.xyz, link), c = -(qxx, qyy, qzz, qxy),
// d = (-qxz, -qyz, m, leaf end). crit = 2 half / theta + |com - centre| (the square root of
// MNode's crit2), negated for a leaf. link (as bits) = first | (children - 1) << 29 for an inner
// node (its children are [first, first + children) in the reference layout), lo for a leaf of
// stars [lo, end).
struct __align__(16) LNode {
    float4 a, b, c, d;
};

// A star's FP64 position and mass in one 32-byte record (one sector per read).
struct __align__(32) Pos4 {
    double x, y, z, m;
};

// Device buffers of the tree path (all owned by the context).
struct TreeBufs {
    int64_t cap_n = 0;      // bodies
    int64_t cap_nodes = 0;  // nodes
    int64_t generation = 0; // incremented whenever the buffers are reallocated
    int32_t group = 64;     // stars per mixed-walk group (32: the list walk, or 64), set before tree_build
    int32_t list_depth = 0; // the list walk's node-list depth (0: kDefaultListDepth), set per call
    // compaction / bbox
    uint32_t *flag = nullptr;     // star flags, then their exclusive scan
    Pos4 *pos4 = nullptr;         // (x, y, z, m) of every star in state order, one 32-byte record
    double *bbox_part = nullptr;  // per-block partial min/max (6 per block)
    // sort
    uint64_t *keys = nullptr, *keys_alt = nullptr;
    int32_t *order = nullptr, *order_alt = nullptr;
    uint32_t *hist = nullptr;     // radix digit table
    // one-sweep sort and single-pass scans: digit histograms, tile counters and look-back words
    // (cleared at the start of every build)
    uint32_t *os_state = nullptr;
    int64_t os_words = 0;
    // larger states: single-pass scans of the three-launch passes' digit tables (a counter and
    // the look-back words of each pass), cleared at each build
    uint32_t *hs_state = nullptr;
    int64_t hs_words = 0;
    // sorted stars
    double *sx = nullptr, *sy = nullptr, *sz = nullptr, *sm = nullptr;
    float4 *st_hi = nullptr, *st_lo = nullptr;
    float4 *st_off = nullptr;  // FP32 offset of each star from its leaf's centre of mass, and its mass
    // chain topology, indexed by sorted position
    uint32_t *chain_cnt = nullptr;  // nodes starting at each position, then the scan
    // pre-order node arrays (index p)
    int32_t *pre_parent = nullptr;
    uint32_t *pre_info = nullptr;   // level | octant << 8
    uint32_t *pre_mask = nullptr;   // occupied child octants (bit per octant)
    uint32_t *pre_nchild = nullptr; // child count, then its exclusive scan
    int32_t *pre_ref = nullptr;     // reference index of pre-order node p
    int32_t *pre_star = nullptr;    // sorted position whose chain holds pre-order node p
    // reference-layout node arrays (index r)
    gbh_node *nodes = nullptr;
    int32_t *n_parent = nullptr;
    uint32_t *n_info = nullptr;     // level | nchild << 8
    int32_t *n_arrive = nullptr;
    PNode *pnodes = nullptr;
    MNode *mnodes = nullptr;
    int2 *mrange = nullptr;
    LNode *lnode = nullptr;         // list-walk records
    uint32_t *walk_ctr = nullptr;   // list walk: next group to take (persistent warps)
    int32_t *leaves = nullptr;      // sorted position of every leaf's first star
    int32_t *targets = nullptr;     // sorted positions of the stars a restricted walk evaluates
    // forest: systems, their geometry, the system of every sorted star, mixed-walk groups
    int32_t nsys = 1;
    int32_t cap_sys = 0;
    SysGeo *geo = nullptr;
    int32_t *sid_sorted = nullptr;  // only when nsys > 1
    int4 *groups = nullptr;         // (first sorted star, count, root, 0); only when nsys > 1
    int64_t cap_groups = 0;
    // Longest-first launch order of the single-system mixed walk: the walk records each group's
    // cost, k_lpt_order turns the costs into the order of the next walk (gperm[cap_groups] = the
    // group count it was made for; any other count means launch order).
    uint32_t *gcost = nullptr;
    int32_t *gperm = nullptr;
    bool lpt = true;                // set per call by the caller
    // Split walks: when a single system has too few 64-star groups to fill the GPU, each group's
    // walk is shared by several warps (parts), each owning a contiguous range of source stars;
    // the parts' sums land in part_acc ([part][axis][cap_n]) and are added in part order.
    double *part_acc = nullptr;
    int64_t part_cap = 0;           // doubles
    bool split = true;              // set per call by the caller
    bool paired = false;            // 64-star groups take the paired walk (set per call)
    int64_t walk_hint = 0;          // a target-list walk's expected list length (0: the body count)
    bool moments_exact = false;     // the last build ran the bit-exact FP64 upsweep
    // scan temporaries
    uint32_t *scan_tmp = nullptr;
    int64_t scan_tmp_cap = 0;
    DevInfo *info = nullptr;
};

// Launch helper context: stream and launch counter.
struct Launch {
    cudaStream_t stream;
    int64_t *count;
    int num_sms;
};

// ---- tree.cu (FP64 parts compiled without FMA contraction) ----
cudaError_t tree_alloc(TreeBufs &b, int64_t n, int leaf_size, int32_t nsys = 1);
void tree_free(TreeBufs &b);
// Builds the tree of the alive non-hole bodies; zeroes alive holes' accelerations. exact:
// FP64 moments bit identical to the reference (the FP64 walk); otherwise the FP32 upsweep of
// moments.cu, which feeds the FP32 walks.
// Forests: sys_of (state order, nsys > 1 only) is each body's system, sys_off (nsys + 1 entries,
// state order) the first body of each system; bodies of a system are contiguous.
cudaError_t tree_build(const Launch &L, TreeBufs &b, int64_t n, const double *px, const double *py,
                       const double *pz, const double *mass, const uint8_t *kind,
                       const uint8_t *alive, double *ax, double *ay, double *az, double theta,
                       int leaf_size, int dm_off, bool exact, bool plain_records = true,
                       const uint16_t *sys_of = nullptr, const int64_t *sys_off = nullptr);
// Block time steps (see tree.cu): tick-0 opening kicks and rungs, drift of all bodies, and the
// closing/opening kicks of the bodies whose step ends at tick. DevInfo.next_tick receives the
// earliest step end over all bodies.
cudaError_t block_open(const Launch &L, const TreeBufs &b, int64_t n, double T, int levels, double eta, double eps,
                       const double *ax, const double *ay, const double *az, double *vx, double *vy, double *vz,
                       uint8_t *rung, int32_t *end);
cudaError_t block_drift(const Launch &L, int64_t n, double dt, double c, double *px, double *py, double *pz, const double *vx,
                        const double *vy, const double *vz);
cudaError_t block_close(const Launch &L, const TreeBufs &b, int64_t n, int32_t tick, double T, int levels, double eta,
                        double eps, const double *ax, const double *ay, const double *az, double *vx, double *vy,
                        double *vz, uint8_t *rung, int32_t *end);
// ---- moments.cu ----
// Every device allocation of the library goes through dev_alloc. A test hook: when a context is
// created with GBH_FAULT_ALLOC=k in the environment, the allocation after the next k successful
// ones fails once with cudaErrorMemoryAllocation (cudaMalloc is not called), so that tests can
// drive the out-of-memory paths from the host; without the variable nothing fails.
cudaError_t dev_alloc_bytes(void **p, size_t bytes);
template <class T>
inline cudaError_t dev_alloc(T **p, size_t bytes) {
    return dev_alloc_bytes(reinterpret_cast<void **>(p), bytes);
}
void arm_alloc_fault(long long after);  // after < 0 disarms

// Parts per group of a split mixed walk over n stars in groups of gsize (1: no split, at most
// 32), from the number of groups per SM.
constexpr int kMaxWalkParts = 32;
int walk_parts(int64_t n, int gsize);
// The most parts a walk sized for n bodies may take (its part_acc budget; 1: never split).
int walk_parts_budget(int64_t n);
// Parts of a split walk (1: none) and the sum of its parts to state order (walk.cu).
int split_parts(const TreeBufs &b, int64_t nstars_cap, bool targets, int gsize);
cudaError_t split_combine(const Launch &L, const TreeBufs &b, int nparts, int64_t stride, bool targets, double *ax,
                          double *ay, double *az);
// Grows part_acc for a split walk over the n bodies of a call (no allocation when it already
// fits). The parts depend on n alone, never on the buffers' capacity, so the same inputs give
// the same bits in any context.
cudaError_t split_reserve(TreeBufs &b, int64_t n);

// FP32 upsweep; writes the walk records of the plain walk (PNode) and/or the mixed walk (MNode).
cudaError_t upsweep_fast(const Launch &L, TreeBufs &b, bool plain_records);
// Test hook (GBH_FAULT_LINK): points the skip link of every leaf that ends its system's walk
// (next == -1) back at node 0 in the node table and in both FP32 walk records, and makes node 0
// that leaf's child for the list walk, so that every walk that reaches that leaf cycles until its
// step bound stops it. Indices stay in range.
cudaError_t fault_link(const Launch &L, TreeBufs &b);
// Fills the FP64 moment fields of the node table from the MNode records (after an FP32 upsweep).
cudaError_t export_fast_moments(const Launch &L, TreeBufs &b);
// Walks: every star, or (targets = true) the stars listed in b.targets (count in DevInfo.ntargets).
cudaError_t walk_fp64(const Launch &L, const TreeBufs &b, int64_t n, double eps2, int quad,
                      double *ax, double *ay, double *az, bool targets = false);
// Lists in b.targets the sorted positions whose body has end[order[k]] == tick.
cudaError_t select_targets(const Launch &L, TreeBufs &b, const int32_t *end, int32_t tick);
cudaError_t kick(const Launch &L, int64_t n, double h, double *vx, double *vy, double *vz,
                 const double *ax, const double *ay, const double *az);
cudaError_t kick_drift(const Launch &L, int64_t n, double h, double dt, double c, double *px, double *py,
                       double *pz, double *vx, double *vy, double *vz, const double *ax,
                       const double *ay, const double *az);
cudaError_t direct_fp64(const Launch &L, int64_t n, const double *px, const double *py,
                        const double *pz, const double *mass, const uint8_t *kind, double eps2,
                        int dm_off, const int64_t *targets, int64_t ntargets, double *ax,
                        double *ay, double *az);
// Potential: psi sums of the FP64 walk plus hole terms; result in *u_dev.
cudaError_t potential_fp64(const Launch &L, const TreeBufs &b, int64_t n, const double *px,
                           const double *py, const double *pz, const double *mass,
                           const uint8_t *kind, const uint8_t *alive, const int32_t *holes,
                           int32_t nholes, double eps2, double c, int dm_off, int quad,
                           double *part, double *u_dev);
// Potential from the mixed walk (FP32 node terms, compensated per-star sums, FP64 reduction);
// psi holds cap_n doubles of scratch. Used for every walk but GBH_WALK_FP64.
cudaError_t potential_mixed(const Launch &L, const TreeBufs &b, int64_t n, const double *px, const double *py,
                            const double *pz, const double *mass, const uint8_t *kind, const uint8_t *alive,
                            const int32_t *holes, int32_t nholes, double eps2, double c, int dm_off, int quad,
                            double *psi, double *part, double *u_dev);
// Exact pair potential of all bodies (PotentialEnergyParallel, diag.go:42-64): rows (n doubles of
// scratch) in ascending i, each over j > i ascending; result in *u_dev.
constexpr int64_t kExactEnergyLimit = 30000;  // exactEnergyLimit, diag.go:16-19
cudaError_t potential_exact_fp64(const Launch &L, int64_t n, const double *px, const double *py, const double *pz,
                                 const double *mass, const uint8_t *kind, double eps2, double c, int dm_off,
                                 double *rows, double *u_dev);
// Sums of diag.go: out[0] kinetic (bodies that gravitate), out[1..3] momentum, out[4..6]
// angular momentum, out[7..9] sum m x, out[10] mass. part holds diag_parts() x 11 doubles.
int diag_parts();
cudaError_t diagnostics(const Launch &L, int64_t n, const double *px, const double *py, const double *pz,
                        const double *vx, const double *vy, const double *vz, const double *mass, const uint8_t *kind,
                        double c, int dm_off, double *part, double *out);
// Exclusive scan of n uint32 in place (in may equal out).
cudaError_t scan_u32(const Launch &L, const uint32_t *in, uint32_t *out, int64_t n,
                     uint32_t *tmp, int64_t tmp_cap);
int64_t scan_tmp_size(int64_t n);

// Stable Morton order of the alive non-hole bodies (collect, keys and radix sort of tree_build)
// with all temporaries in one caller-provided device block of scratch_bytes; keys/order get the
// sorted keys and state indices, *info_out points at the DevInfo inside the block.
size_t morton_sort_scratch_bytes(int64_t nmax);
cudaError_t morton_sort(const Launch &L, int64_t n, const double *px, const double *py, const double *pz,
                        const uint8_t *kind, const uint8_t *alive, uint64_t *keys, int32_t *order, void *scratch,
                        size_t scratch_bytes, DevInfo **info_out);

// ---- split.cu (the hole-aware step of split.go with c = 0) ----
struct SplitBufs {
    int32_t *holes = nullptr;  // alive holes, ascending state index
    int32_t nholes = 0, cap_holes = 0;
    uint8_t *near8 = nullptr;   // near flags
    uint32_t *near32 = nullptr; // near flags, then their exclusive scan
    int32_t *near = nullptr;    // near stars, ascending
    uint32_t *scan_tmp = nullptr;
    int64_t scan_cap = 0;
    double *far = nullptr, *fast = nullptr;  // 3n each (x, y, z blocks)
    double *part = nullptr;                  // per 256-body chunk and hole: 3 partial sums
    int64_t cap_n = 0, cap_part = 0;
    unsigned long long *scalars = nullptr;   // [0] bits of the minimum timescale, [1] near count
};
cudaError_t split_reserve(SplitBufs &s, int64_t n, const std::vector<int32_t> &holes);
void split_free(SplitBufs &s);
// Near flags and list, minimum timescale (scalars) for the current positions.
cudaError_t split_classify(const Launch &L, SplitBufs &s, int64_t n, const double *px, const double *py,
                           const double *pz, const double *mass, const uint8_t *kind, double eps2, double c,
                           double limit);
// far = hole pulls of the far stars and the far stars' pulls on the holes.
cudaError_t split_outer(const Launch &L, SplitBufs &s, int64_t n, const double *px, const double *py,
                        const double *pz, const double *mass, const uint8_t *kind, int dm_off, double eps2, double c);
cudaError_t split_kick_outer(const Launch &L, SplitBufs &s, int64_t n, double h, double *vx, double *vy, double *vz,
                             const double *ax, const double *ay, const double *az);
// fast = hole pulls of the near stars, and the holes' pulls from the other holes and the near stars.
cudaError_t split_fast(const Launch &L, SplitBufs &s, int64_t n, int32_t nnear, const double *px, const double *py,
                       const double *pz, const double *mass, const uint8_t *kind, int dm_off, double eps2, double c);
// Near stars and holes: v += h fast (drift = false) or x += h v (drift = true).
cudaError_t split_fast_update(const Launch &L, SplitBufs &s, int64_t n, int32_t nnear, bool drift, double h,
                              double c, double *px, double *py, double *pz, double *vx, double *vy, double *vz);
cudaError_t split_drift_far(const Launch &L, SplitBufs &s, int64_t n, double dt, double c, const uint8_t *kind,
                            double *px, double *py, double *pz, const double *vx, const double *vy, const double *vz);

// ---- adjoint.cu (gradient of the KDK leapfrog with the softened direct-sum force) ----
// Scratch of the tree adjoint (walk_lists.cu): node-moment and source-star accumulators, each
// sorted star's own terms and its leaf.
struct AdjTreeBufs {
    double *nadj = nullptr, *sadj = nullptr, *tgt = nullptr;
    int32_t *star_leaf = nullptr;
    int64_t cap_nodes = 0, cap_n = 0;
};

struct AdjTape {
    void *block = nullptr;  // one grow-only allocation holding every array below
    size_t bytes = 0;
    int64_t n = 0, nsteps = 0, every = 1, nck = 0, chunk = 0;
    int nsplit = 1;
    double dt = 0, eps2 = 0;
    bool fp32 = false, valid = false;
    double *x = nullptr, *v = nullptr, *a = nullptr;  // 3n each: the working state (x_T after the forward)
    double *m = nullptr;                              // n
    double *lam = nullptr;                            // 7n: lambda_x (3n), lambda_v (3n), lambda_m (n)
    double *ck = nullptr;                             // nck x 9n: (x, v, a) at steps 0, K, 2K, ...
    double *seg = nullptr;                            // K x 3n: positions of one replayed segment
    double *rv = nullptr, *ra = nullptr;              // 3n each: velocities and accelerations of the replay
    double *part = nullptr;                           // nsplit x 4n: FP32 pair sums per source split
    float4 *hi = nullptr, *lo = nullptr, *w = nullptr;  // n each: FP32 positions + mass, remainders, weights
    // Tree force (gbh_adjoint_params.force = GBH_ADJ_TREE): the list walk in 32-star groups at
    // theta and leaf size leaf, on the context's tree buffers, and the adjoint's own scratch.
    bool tree = false;
    double theta = 0.9;
    int leaf = 24;
    TreeBufs *tb = nullptr;
    AdjTreeBufs tbs;
    // Optional stage marks around each pair-kernel launch: (prep start, pair start, pair end).
    cudaError_t (*mark)(void *) = nullptr;
    void *mark_arg = nullptr;
};
// Carves the tape for n bodies, nsteps steps and checkpoints every `every` steps (grow-only).
cudaError_t adj_reserve(AdjTape &t, int64_t n, int64_t nsteps, int64_t every, double dt, double eps, bool fp32,
                        int num_sms);
void adj_free(AdjTape &t);
// nsteps KDK steps from (t.x, t.v) with masses t.m, saving checkpoints; leaves x_T, v_T in t.x, t.v.
cudaError_t adj_forward(const Launch &L, AdjTape &t);
// From t.lam = (dL/dx_T, dL/dv_T, 0) to (dL/dx_0, dL/dv_0, dL/dm) in place.
cudaError_t adj_backward(const Launch &L, AdjTape &t);

// ---- walk.cu (FP32 walks, FMA contraction on) ----
cudaError_t walk_plain(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2,
                       double *ax, double *ay, double *az, bool targets = false);
cudaError_t walk_mixed(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2,
                       int quad, double *ax, double *ay, double *az, bool targets = false);
// psi[k] = sum m / r + (d.Q.d) / (2 r^5) of sorted star k (walkPotential with the mixed walk).
cudaError_t walk_mixed_potential(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, int quad,
                                 double *psi);
cudaError_t fp32_fma_probe(const Launch &L, int blocks, int iters, float *out);
// Longest-first order of the next walk's groups of gsize stars, from this walk's group costs.
cudaError_t lpt_order(const Launch &L, const TreeBufs &b, int gsize);

// ---- walk_lists.cu (the list walk: decoupled traversal and evaluation, 32- or 64-star groups) ----
constexpr int kDefaultListDepth = 56;
// The largest node-list depth (entries evaluated per flush) of the list walk.
int list_depth_max(bool exact);
// Every star, or (targets = true) the stars listed in b.targets, in groups of 32 x stars_per_lane
// (1 or 2) stars; a forest's build must have made groups of that size (b.group). Persistent
// warps; needs b.cap_nodes < 2^29. With few groups for the GPU (b.split, split_parts) each group's
// walk is shared among several warps; nstars_cap (>= the body count) is then the stride of the
// part accumulators.
cudaError_t walk_lists(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, int quad, double *ax,
                       double *ay, double *az, int list_depth, bool targets, int stars_per_lane);
// psi of every star by sorted index (the tree potential of potential.go:44-81) with the list walk:
// 64-star groups of the build (b.group == 64), softening > 0, b.cap_nodes < 2^29.
cudaError_t walk_lists_potential(const Launch &L, const TreeBufs &b, float eps2, int quad, double *psi);
// The transposed Jacobian of the list walk's force (the groups of b.group, quadrupoles, softening > 0)
// with the lists of the tree in b frozen: for weights w (state order) writes, in state order,
// (J^T w)_i and (da/dm)^T w_i into out (x, y, z and m terms, n apart). px .. mass: the state the
// tree was built from.
cudaError_t walk_lists_adjoint(const Launch &L, const TreeBufs &b, float eps2, const double *px, const double *py,
                               const double *pz, const double *mass, const double *wx, const double *wy,
                               const double *wz, int64_t n, AdjTreeBufs &s, double *out);
cudaError_t adj_tree_reserve(AdjTreeBufs &s, const TreeBufs &b);
void adj_tree_free(AdjTreeBufs &s);

}  // namespace gbh
