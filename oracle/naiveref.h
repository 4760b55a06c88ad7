/*
 * naiveref.h -- CPU oracle for the NaiveDynamics.jl neighbour-search / force /
 * integrator hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates the reference algorithm in
 * plain C so that the GPU library can be checked against it.  Only the test
 * suite, the smoke check and the benchmark's CPU-baseline leg may load it; the
 * product path (libnaivegpu) never links or calls it.
 *
 * Conventions follow the reference (Julia, 1-based):
 *   - node indices in keys (left, skip) are 1-based, 0 is the sentinel;
 *   - leaves are nodes 1..nL, internal node k (1..nL-1) is node nL+k,
 *     the root is node nL+1;
 *   - atom indices written into pair lists are the 1-based ORIGINAL indices.
 * Every function cites the reference file:line it restates.
 */
#ifndef NAIVEREF_H
#define NAIVEREF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define REF_OK             0
#define REF_ERR_ARG       -1
#define REF_ERR_SPEC      -2
#define REF_ERR_NONFINITE -3
#define REF_ERR_RANGE     -4
#define REF_ERR_NOMEM     -6

/* GridKey{Float32,Int32} (src/Neighbors/BVHTraverse.jl:102-109): 32 bytes. */
typedef struct {
    float min[3];
    float max[3];
    int32_t left;
    int32_t skip;
} ref_key;

/* Ordering of atoms before the tree build. */
#define REF_ORDER_REFERENCE 0 /* mortoncodes! bit-select code (BVHTraverse.jl:237-288) */
#define REF_ORDER_SPATIAL   1 /* 3-D Hilbert index, 10 bits per axis over the bounding box */

/* Leaf bounding boxes. */
#define REF_BOX_LEAF 0 /* leafcluster_primitives: p -/+ r/2, key array N-1 (BVHTraverse.jl:376-410) */
#define REF_BOX_ATOM 1 /* cluster_primitives:     p -/+ r,   key array 2nL-1 (BVHTraverse.jl:341-375) */

/* SpheresBVHSpecs constructor checks (BVHTraverse.jl:71-94). */
int ref_spec(int64_t atom_count, int64_t atomsperleaf, int32_t* leaves, int32_t* branches);

/* mortoncodes! for K = Int32 (BVHTraverse.jl:237-288) with binwidth = Float32(1/1023) (:184). */
int ref_morton_reference(const float* xyz, int64_t n, int32_t* codes);

/* Spatial code: 3-D Hilbert index, 10 bits per axis over the bounding box. */
int ref_morton_spatial(const float* xyz, int64_t n, int32_t* codes);
uint32_t ref_hilbert3(uint32_t x, uint32_t y, uint32_t z);

/* Stable ascending sortperm (BVHTraverse.jl:570); perm is 0-based. */
int ref_sortperm(const int32_t* codes, int64_t n, int32_t* perm);

/* exptdelta (BVHTraverse.jl:677-696), i is the 1-based leaf index. */
int32_t ref_delta(int32_t i, const int32_t* code_sorted, int32_t nL, int32_t apl);

/*
 * leafTreeData (BVHTraverse.jl:544-597) when boxes == REF_BOX_LEAF,
 * TreeData (BVHTraverse.jl:500-543) when boxes == REF_BOX_ATOM.
 * keys must hold nkeys entries (N-1 for REF_BOX_LEAF -- apl must be >= 2 there,
 * as the reference indexes past N-1 otherwise -- and 2nL-1 for REF_BOX_ATOM).
 * idx_sorted: 1-based original index per sorted atom; code_sorted: Morton code
 * per sorted atom; pos_sorted: N*3 floats; perm: 0-based sortperm.
 * overwrite_root: 1 replays the root box overwrite of BVHTraverse.jl:856-858.
 */
int ref_tree(const float* xyz, int32_t n, float r, int32_t apl, int32_t order, int32_t boxes,
             int32_t overwrite_root, ref_key* keys, int64_t nkeys, int32_t* idx_sorted,
             int32_t* code_sorted, float* pos_sorted, int32_t* perm);

/* The leafTreeData tree (leaf boxes p -/+ r/2) of positions xyz in a kept
 * order: idx_sorted (1-based original index per sorted slot) and code_sorted
 * from an earlier ref_tree; the same topology with the new boxes. */
int ref_tree_kept(const float* xyz, int32_t n, float r, int32_t apl, int32_t overwrite_root,
                  ref_key* keys, int64_t nkeys, const int32_t* idx_sorted,
                  const int32_t* code_sorted, float* pos_sorted);

/*
 * leafneighbor_traverse (BVHTraverse.jl:1236-1323) run with one thread: emits
 * pairs in the reference's serial order.  Returns the number of pairs; writes
 * at most cap of them (pi/pj/pd may be NULL when cap == 0).
 */
int64_t ref_leaf_traverse(const ref_key* keys, const int32_t* idx_sorted, const float* pos_sorted,
                          int32_t nL, int32_t apl, float r, int32_t* pi, int32_t* pj, float* pd,
                          int64_t cap);
/* The same traversal with a pair criterion: 0 = d^2 < r^2 (leafneighbor_traverse),
 * 1 = sqrt(d^2) < r (simdneighbor_traverse, ext/NaiveSIMD.jl:529,589). */
int64_t ref_leaf_traverse_crit(const ref_key* keys, const int32_t* idx, const float* pos,
                               int32_t nL, int32_t apl, float r, int32_t criterion, int32_t* pi,
                               int32_t* pj, float* pd, int64_t cap);

/* Same traversal, counting and hashing only, OpenMP over query leaves. */
int64_t ref_leaf_traverse_hash(const ref_key* keys, const int32_t* idx_sorted,
                               const float* pos_sorted, int32_t nL, int32_t apl, float r,
                               uint64_t hash_out[2]);

/* neighbor_traverse (BVHTraverse.jl:1125-1183), per-atom traversal made runnable. */
int64_t ref_atom_traverse(const ref_key* keys, const int32_t* idx_sorted, const float* pos_sorted,
                          int32_t n, int32_t apl, float r, int32_t* pi, int32_t* pj, float* pd,
                          int64_t cap);

/*
 * unique_pairs + threshold_pairs (src/Neighbors/AllToAll.jl:65-88).
 * criterion 0: d^2 < r^2 (the leaf-BVH test, BVHTraverse.jl:1048);
 * criterion 1: sqrt(d^2) < r (AllToAll.jl:86, ext/NaiveSIMD.jl:529,589).
 * Pairs (i, j) with i < j, 1-based, in lexicographic order.
 */
/* Bug-compatible force_lennardjones! / force_coulomb! (Forces.jl:6-66): the
 * list in order, Float32 accumulators, force N x 3 (zeroed first). */
void ref_compat_force_lj(int32_t n, const int32_t* pi, const int32_t* pj, const float* pd,
                         int64_t np, float* force);
void ref_compat_force_coulomb(int32_t n, const int32_t* pi, const int32_t* pj, const float* pd,
                              int64_t np, const float* q, float* force);

/* simulate! as written (Simulator.jl:154-256), Float32 state, Int64
 * stepwidth; the layout of the spec matches the library's nd_compat_sim.
 * poslog: NULL or (duration + 1) x n x 3.  Returns 0, or 1 when
 * rescale_velocity! raises Julia's DomainError (state as at the throw). */
typedef struct ref_compat_sim {
    float min_dim[3];
    float max_dim[3];
    float temperature;
    int64_t objectnumber;
    int64_t stepwidth;
    int64_t duration;
    float velocity_dampening;
} ref_compat_sim;
int ref_compat_simulate(const ref_compat_sim* spec, int32_t n, float* x, float* v, float* force,
                        const float* mass, const float* q, float* poslog);

/* collect_objects (MDInput.jl:305-369) with the library's counter-based
 * stream (layout matches nd_collector); unique_pairs_prune's loop run
 * literally.  Returns the number of atoms filled with Inf. */
typedef struct ref_collector {
    int64_t objectnumber;
    float min_dim[3];
    float max_dim[3];
    float temperature;
    int32_t randomvelocity;
    float minmass;
    float maxmass;
    float minimumdistance;
    float mincharge;
    float maxcharge;
} ref_collector;
int64_t ref_collect_objects(const ref_collector* cl, uint64_t seed, float* x, float* v, float* m,
                            float* q);

int64_t ref_brute_pairs(const float* xyz, int32_t n, float r, int32_t criterion, int32_t* pi,
                        int32_t* pj, float* pd, int64_t cap);

/* Squared distance exactly as sum((a - b).^2) on SVector{3,Float32}. */
float ref_dist2(const float* a, const float* b);

/* Order-free 128-bit hash of canonical (min(i,j), max(i,j), bits(d)) triples. */
void ref_pair_hash(const int32_t* pi, const int32_t* pj, const float* pd, int64_t np,
                   uint64_t hash_out[2]);

/* ---------------------------------------------------------------- physics (FP64) */

typedef struct {
    double sigma, epsilon;   /* Lennard-Jones */
    double coulomb_k;        /* Coulomb constant, 0 disables */
    double cutoff;           /* force cutoff */
    double box_lo[3];        /* reflecting walls, boundary_reflect! (Simulator.jl:81-111) */
    double box_hi[3];
    double dt;
} ref_md_params;

/*
 * Truncated LJ + cutoff Coulomb forces and potential energy over all pairs with
 * r < cutoff, found with a cell list (independent of the BVH).  x: N*3, q: N
 * (may be NULL when coulomb_k == 0), f: N*3 out, energy: out (may be NULL).
 * Returns the number of interacting pairs.
 */
int64_t ref_forces(const ref_md_params* p, int32_t n, const double* x, const double* q,
                   double* f, double* energy);

/* Ensemble checks call ref_forces / ref_md_run once per system (systems are
 * independent), with that system's sigma, epsilon and walls. */

/*
 * Kick-drift-kick velocity Verlet with reflecting walls:
 *   v += dt/2 F/m; x += dt v; reflect; F = F(x); v += dt/2 F/m
 * f must hold F(x) on entry (computed by ref_forces) and holds F(x) on exit.
 * m may be NULL (unit masses).
 */
int ref_md_run(const ref_md_params* p, int32_t n, double* x, double* v, double* f,
               const double* q, const double* m, int64_t steps);

/*
 * ref_md_run with the step loop's observers of simulate! (Simulator.jl:241-245):
 * after every thermo_every-th step rescale_velocity! (Simulator.jl:119-144)
 * with temperature thermo_T and damping thermo_gamma (0 = off), and after
 * every log_every-th step the positions appended to poslog (frames x N x 3;
 * 0 or poslog NULL = off).
 */
int ref_md_run_observed(const ref_md_params* p, int32_t n, double* x, double* v, double* f,
                        const double* q, const double* m, int64_t steps, double thermo_T,
                        double thermo_gamma, int32_t thermo_every, int32_t log_every,
                        double* poslog);

/*
 * CPU baseline: the reference path timed on host cores.  Every `rebuild`
 * steps the leaf BVH (reference order, leafTreeData + leafneighbor_traverse)
 * is rebuilt at radius cutoff + skin from Float32 positions; forces are
 * evaluated over that half pair list in FP64 with OpenMP.  Returns pairs of
 * the last list, or a negative status.
 */
int64_t ref_md_run_bvh(const ref_md_params* p, int32_t n, double* x, double* v, double* f,
                       const double* q, const double* m, int64_t steps, int32_t rebuild,
                       double skin, int32_t apl, int32_t order);

int ref_num_threads(void);

/*
 * The same loop as a session, for timing steady-state windows: create copies
 * x, v (N x 3), q, m (either may be NULL), builds the first list and evaluates
 * the forces; steps advances, rebuilding after every `rebuild`-th step since
 * creation (so `rebuild` steps hold one build), and returns the pairs of the
 * current list or a negative status.  NULL from create: bad input or no memory.
 */
typedef struct ref_md_bvh ref_md_bvh;
ref_md_bvh* ref_md_bvh_create(const ref_md_params* p, int32_t n, const double* x,
                              const double* v, const double* q, const double* m,
                              int32_t rebuild, double skin, int32_t apl, int32_t order);
int64_t ref_md_bvh_steps(ref_md_bvh* s, int64_t steps);
void ref_md_bvh_get(const ref_md_bvh* s, double* x, double* v, double* f);
void ref_md_bvh_destroy(ref_md_bvh* s);

/*
 * Seeded synthetic inputs of the benchmark workloads (splitmix64 stream):
 * uniform Float32 positions in [lo, lo + side)^3; FP64 positions in
 * [0, side)^3 with no two closer than dmin (random sequential addition);
 * N(0, s^2) values; charges +1 / -1, half each, shuffled.  Status 0 or
 * negative.
 */
int ref_synth_uniform(uint64_t seed, int32_t n, double lo, double side, float* xyz);
int ref_synth_uniform_mindist(uint64_t seed, int32_t n, double side, double dmin, double* xyz);
int ref_synth_normal(uint64_t seed, int64_t count, double s, double* out);
int ref_synth_charges(uint64_t seed, int32_t n, double* q);

/* ------------------------------------------------ differentiable trajectory */

/* Loss of a trajectory: steps of kick-drift-kick, then the Gaussian-smoothed
 * pair-distance histogram of the final positions (bins on [0, r_max], width
 * `width`, pair weights switched to 0 between r_switch and r_max) against a
 * target, L = sum_b (h_b - target_b)^2.  See naiveadj.c. */
typedef struct {
    int32_t steps;
    int32_t bins;
    double r_max;
    double width;
    double r_switch;
} ref_adj_spec;

/*
 * Forward-mode (dual-number) evaluation of the loss: value and its derivatives
 * dloss[0] = dL/dsigma, dloss[1] = dL/depsilon, dloss[2] = the directional
 * derivative along (dx0, dv0) (either may be NULL = 0).  target may be NULL
 * (zeros).  hist (bins), x_out, v_out (N x 3), events (2) may be NULL.
 */
int ref_adj_dual(const ref_md_params* p, const ref_adj_spec* s, int32_t n, const double* x0,
                 const double* v0, const double* q, const double* m, const double* dx0,
                 const double* dv0, const double* target, double* hist, double* loss,
                 double dloss[3], double* x_out, double* v_out, uint64_t events[2]);

#ifdef __cplusplus
}
#endif
#endif
