/*
 * bh_oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement, in C++, of gravitas' Barnes-Hut quadrupole force path
 * (internal/sim/bh/{morton,parallel,build,bh,potential}.go), its FP64 direct
 * sum (internal/sim/direct/direct.go) and its KDK leapfrog
 * (internal/sim/sim.go). It is the parity oracle for the CUDA library and the
 * timed CPU baseline; it is never linked into, or called by, the product path.
 * Only tests/, __graft_entry__.smoke() and bench.py (its CPU baseline legs)
 * load it.
 *
 * Floating point: compiled with -ffp-contract=off, so every a*b+c is a rounded
 * multiply followed by a rounded add, as the Go compiler emits on amd64. (Go on
 * arm64 fuses some of them into FMAs, so the reference itself differs in the
 * last bits between platforms; the no-fusion semantics are the ones pinned.)
 */
#ifndef GRAVITAS_BH_ORACLE_H
#define GRAVITAS_BH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors internal/sim/bh/bh.go:59-67 (type node). */
typedef struct {
    double x, y, z, m;
    double qxx, qyy, qzz, qxy, qxz, qyz;
    double crit2;
    int32_t first, next, lo, hi;
} orc_node;

/* Body kinds, internal/sim/state.go:12-21. */
enum { ORC_STAR = 0, ORC_BLACK_HOLE = 1, ORC_DARK_MATTER = 2, ORC_GAS = 3 };

/* morton.go:19-21. */
uint64_t orc_morton_key(uint64_t x, uint64_t y, uint64_t z);
/* morton.go:25-49 (serial stable LSD radix sort, 8-bit digits). */
void orc_radix_sort(uint64_t *keys, int32_t *idx, int64_t n);
/* parallel.go:33-88 (per-worker histograms, static chunks). */
void orc_radix_sort_parallel(uint64_t *keys, int32_t *idx, int64_t n, int workers);

/* A built tree: sorted stars plus the node table. */
typedef struct orc_tree orc_tree;
orc_tree *orc_tree_new(void);
void orc_tree_free(orc_tree *t);

/*
 * build.go:11-51. Builds the tree for the alive non-hole bodies. workers <= 0
 * means all hardware threads; workers == 1 gives the serial build whose node
 * indices are the canonical layout (buildParallel gives the same forces with a
 * different index layout, build.go:219-296). Returns the node count.
 */
int64_t orc_tree_build(orc_tree *t, int64_t n, const double *px, const double *py,
                       const double *pz, const double *mass, const uint8_t *kind,
                       const uint8_t *alive, double theta, int leaf_size,
                       int dark_matter_off, int workers);
int64_t orc_tree_nstars(const orc_tree *t);
int64_t orc_tree_nnodes(const orc_tree *t);
int64_t orc_tree_nholes(const orc_tree *t);
/* Root cube: min corner and side (build.go:19-21, 43-50). */
void orc_tree_box(const orc_tree *t, double *min3, double *side);
/* Any pointer may be NULL. keys/order/sx..sm have nstars entries, nodes nnodes. */
void orc_tree_export(const orc_tree *t, uint64_t *keys, int32_t *order, orc_node *nodes,
                     double *sx, double *sy, double *sz, double *sm, int32_t *holes);

/*
 * bh.go:76-102 + walk bh.go:106-155: accelerations in state order (n =
 * the state length passed to build), holes and dead bodies get 0.
 */
void orc_tree_accelerations(const orc_tree *t, int64_t n, double eps, int monopole_only,
                            int workers, double *ax, double *ay, double *az);
/* walk bh.go:106-155 for one point; self = sorted index to skip or -1. */
void orc_tree_walk_point(const orc_tree *t, double x, double y, double z, int32_t self,
                         double eps2, int monopole_only, double *a3);
/* walkPotential potential.go:45-81 for one point. */
double orc_tree_walk_potential_point(const orc_tree *t, double x, double y, double z,
                                     int32_t self, double eps2, int monopole_only);
/*
 * Interaction counts of the reference per-target walk for the sorted targets
 * listed (all targets if targets == NULL): accepted nodes, leaf star pairs and
 * opened nodes. These are the counts behind the algorithmic FLOP figure.
 */
void orc_tree_counts(const orc_tree *t, double eps, int monopole_only, int workers,
                     const int32_t *targets, int64_t ntargets, int64_t *n_node,
                     int64_t *n_pp, int64_t *n_open);
/*
 * Counts of the group walk that the GPU mixed walk executes: groups of `group` consecutive
 * sorted stars open a node when any of their stars would; every star takes part in each of its
 * group's visits. Summed over stars with the definitions of orc_tree_counts (group = 1 gives
 * the per-star counts).
 */
void orc_tree_group_counts(const orc_tree *t, int group, int workers, int64_t *n_node,
                           int64_t *n_pp, int64_t *n_open);
/*
 * The float32 Metal walk (internal/sim/bh/gpu_darwin.go:84-117, nodes packed as
 * :187-202) restated on the CPU. Output in sorted order, 3 floats per star.
 */
void orc_tree_walk_fp32(const orc_tree *t, double eps, int workers, float *acc3_sorted);

/*
 * potential.go:12-42: U from the tree walk (theta is the caller's choice; the
 * reference passes min(theta, 0.9)). Star–hole and hole–hole pairs use the
 * pair model with speed of light c (pair.go).
 */
double orc_tree_potential(const orc_tree *t, int64_t n, const double *px, const double *py,
                          const double *pz, const double *mass, const uint8_t *kind,
                          const uint8_t *alive, double eps, double c, int dark_matter_off,
                          int monopole_only, int workers);

/* direct.go:18-48: O(N^2) FP64 star–star accelerations, holes get 0. */
void orc_direct(int64_t n, const double *px, const double *py, const double *pz,
                const double *mass, const uint8_t *kind, double eps, int dark_matter_off,
                int workers, double *ax, double *ay, double *az);
/* Direct sum for a subset of targets (state indices); out has ntargets rows. */
void orc_direct_targets(int64_t n, const double *px, const double *py, const double *pz,
                        const double *mass, const uint8_t *kind, double eps,
                        int dark_matter_off, const int64_t *targets, int64_t ntargets,
                        int workers, double *ax, double *ay, double *az);

/*
 * sim.go:252-288 with no holes and no gas: nsteps KDK steps with the
 * Barnes-Hut solver (drift sim.go:315-343: x += dt v for c <= 0, x += dt u / gamma for c > 0). Forces at entry are taken
 * from acc when acc_valid, else computed first (initForces, gas.go:14-17).
 * Arrays are updated in place.
 */
void orc_kdk(int64_t n, double *px, double *py, double *pz, double *vx, double *vy,
             double *vz, double *ax, double *ay, double *az, const double *mass,
             const uint8_t *kind, const uint8_t *alive, double dt, double eps, double theta,
             int leaf_size, int monopole_only, int dark_matter_off, int acc_valid,
             int64_t nsteps, int workers, double c);

/*
 * Block time steps for gravity, on the scheme of the reference's gas block steps
 * (internal/sim/blockstep.go:22-90; gravity itself has no block steps in the reference):
 * rung r = smallest with dt/2^r <= eta*sqrt(eps/|a|) (rungFor, blockstep.go:38-45), capped at
 * levels-1, steps start at multiples of their length (blockstep.go:84-86), per-body KDK, all
 * bodies drift from event to event, tree rebuilt at each event, only bodies whose step ends
 * are walked and kicked. Counts of events and walked stars go to *substeps / *evals.
 */
void orc_block_kdk(int64_t n, double *px, double *py, double *pz, double *vx, double *vy,
                   double *vz, double *ax, double *ay, double *az, const double *mass,
                   const uint8_t *kind, const uint8_t *alive, double dt, double eta, int levels,
                   double eps, double theta, int leaf_size, int monopole_only, int dark_matter_off,
                   int acc_valid, int64_t nsteps, int workers, int64_t *substeps, int64_t *evals,
                   double c);

/*
 * The hole-aware step of internal/sim/split.go:1-259 (stepSplit) without gas, with the pair model
 * of pair.go:26-35 (Paczynski-Wiita star-hole forces for c > 0) and the drift of u / gamma, but
 * with instant gravity, no frame dragging (no spins) and no accretion or collapse (those follow
 * the step in sim.go:260-287 and are not restated): star-star forces from the tree once per step; every force involving an alive
 * black hole summed directly; stars whose timescale at a hole is below 20 dt ("near") and the
 * holes take n power-of-two substeps (classify, split.go:39-85). Steps without holes are the
 * plain KDK of orc_kdk. A hole's pull from the far stars is summed in chunks of 256 bodies
 * (sequential inside a chunk, chunks in index order); the reference sums its ParallelFor chunks
 * in completion order, so its last bits vary from run to run there. *substeps gets n of the
 * last step and near (n bytes, may be NULL) its near flags.
 */
void orc_split_kdk(int64_t n, double *px, double *py, double *pz, double *vx, double *vy,
                   double *vz, double *ax, double *ay, double *az, const double *mass,
                   const uint8_t *kind, const uint8_t *alive, double dt, double eps, double theta,
                   int leaf_size, int monopole_only, int dark_matter_off, int acc_valid,
                   int64_t nsteps, int workers, int64_t *substeps, uint8_t *near, double c);

/*
 * Adjoint of the KDK leapfrog (sim.go:302-343) with the softened direct-sum force
 * (direct.go:27-47, all bodies stars): the gradient of a loss with respect to the initial
 * positions, velocities and masses, given its gradient (gx.., gv..) with respect to the final
 * positions and velocities after nsteps steps of dt from the state (x0, v0). FP64. The forward
 * trajectory is replayed from checkpoints every `every` steps. No counterpart in the
 * reference: the oracle of gbh_fwd_save / gbh_bwd.
 */
void orc_adjoint_direct(int64_t n, const double *px, const double *py, const double *pz,
                        const double *vx, const double *vy, const double *vz, const double *mass,
                        double eps, double dt, int64_t nsteps, int64_t every, const double *gx,
                        const double *gy, const double *gz, const double *gvx, const double *gvy,
                        const double *gvz, double *dx, double *dy, double *dz, double *dvx,
                        double *dvy, double *dvz, double *dm, int workers);
/* The forward of orc_adjoint_direct: nsteps KDK steps with the direct-sum force, in place. */
void orc_kdk_direct(int64_t n, double *px, double *py, double *pz, double *vx, double *vy,
                    double *vz, const double *mass, double eps, double dt, int64_t nsteps,
                    int workers);

/* The pair model (pair.go:14-47): PairForce, PairPotential, PairRS. */
double orc_pair_force(double m, double r2, double eps2, double rs);
double orc_pair_potential(double mi, double mj, double r2, double eps2, double rs);
double orc_pair_rs(uint8_t ki, double mi, uint8_t kj, double mj, double c);

/* diag.go:44-64 exact pair potential (no holes: plain softened Newtonian). */
double orc_potential_exact(int64_t n, const double *px, const double *py, const double *pz,
                           const double *mass, const uint8_t *kind, double eps, double c,
                           int dark_matter_off, int workers);

#ifdef __cplusplus
}
#endif
#endif
