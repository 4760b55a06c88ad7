/*
 * naivegpu.h -- C ABI of libnaivegpu, the GB300 (sm_103a) implementation of the
 * NaiveDynamics.jl per-step hot path:
 *
 *   LBVH neighbour search   (src/Neighbors/BVHTraverse.jl)
 *   LJ + Coulomb forces     (src/Forces.jl)
 *   velocity-Verlet update  (src/Simulator.jl)
 *
 * It replaces the package-extension backends ext/NaiveKA.jl and ext/NaiveCUDA.jl
 * behind the extension seam of src/PkgExtensions.jl.  Every entry point cites
 * the reference function it replaces.
 *
 * Conventions
 *   - Every function returns an nd_status (0 = ND_OK) and never throws or aborts.
 *   - Plain pointers are HOST pointers unless the function name ends in _dev,
 *     in which case they are device pointers on the context's device and the
 *     work is enqueued on the context's stream.
 *   - Atom indices written to pair lists are 1-based ORIGINAL indices and tree
 *     node indices (left, skip) are 1-based with 0 as the sentinel, exactly as in
 *     the reference (Julia) data structures.
 *   - Positions for neighbour search are Float32, x y z interleaved (N x 3), the
 *     memory layout of Vector{MVector{3,Float32}} (src/MDInput.jl:29).
 *   - One context = one device = one stream; a context is not thread-safe.
 */
#ifndef NAIVEGPU_H
#define NAIVEGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t nd_status;

#define ND_OK              0
#define ND_NEED_REALLOC    1  /* output buffer too small; the needed count is returned */
#define ND_ERR_ARG        -1  /* bad argument (NULL pointer, negative size, ...)       */
#define ND_ERR_SPEC       -2  /* SpheresBVHSpecs checks (BVHTraverse.jl:74-80)           */
#define ND_ERR_NONFINITE  -3  /* NaN/Inf coordinate: InexactError of round(Int32, ...) */
#define ND_ERR_RANGE      -4  /* p/binwidth outside Int32 (BVHTraverse.jl:266)         */
#define ND_ERR_CUDA       -5  /* CUDA runtime error; nd_last_error() has the message    */
#define ND_ERR_NOMEM      -6  /* device allocation failed                               */
#define ND_ERR_INTERNAL   -7  /* device-side consistency check failed (error flag)      */
#define ND_ERR_OVERFLOW   -8  /* neighbour list capacity exceeded during a run          */
#define ND_ERR_NODEVICE   -9  /* no CUDA device / device index out of range             */

/* Atom ordering before the tree build. */
#define ND_ORDER_REFERENCE 0  /* mortoncodes! bit-select code, bit-exact with the reference */
#define ND_ORDER_SPATIAL   1  /* 3-D Hilbert index, 10 bits/axis over the bounding box      */

/* Leaf boxes. */
#define ND_BOX_LEAF 0  /* leafcluster_primitives: p -/+ r/2 (BVHTraverse.jl:376-410) */
#define ND_BOX_ATOM 1  /* cluster_primitives:     p -/+ r   (BVHTraverse.jl:341-375) */

/* Pair-list emission order. */
#define ND_PAIRS_ORDERED   0  /* exactly the reference's single-thread emission order */
#define ND_PAIRS_UNORDERED 1  /* same multiset, order decided at run time (one pass)  */

/* Pair criterion on the Float32 squared distance d2 (d = sqrt(d2), rounded). */
#define ND_CRIT_SQUARED 0  /* d2 < r^2: leafneighbor_traverse (BVHTraverse.jl:1048)        */
#define ND_CRIT_SQRT    1  /* d < r: simdneighbor_traverse (ext/NaiveSIMD.jl:529,589)      */

typedef struct nd_ctx nd_ctx;
typedef struct nd_md nd_md;

/* SpheresBVHSpecs{Float32,Int32} (BVHTraverse.jl:63-69). */
typedef struct {
    float neighbor_distance;
    int32_t atom_count;
    int32_t leaves_count;
    int32_t branches_count;
    int32_t atomsperleaf;
} nd_bvh_spec;

/* GridKey{Float32,Int32} (BVHTraverse.jl:102-109), 32 bytes. */
typedef struct {
    float min[3];
    float max[3];
    int32_t left;
    int32_t skip;
} nd_gridkey;

/* Force model and integrator parameters: the keywords the reference hard-codes
 * (Forces.jl:17-19,57) plus SimSpec.stepwidth (Simulator.jl:30-49) and the
 * GenericRandomCollector walls minDim/maxDim (MDInput.jl:67-84). */
typedef struct {
    double sigma;
    double epsilon;
    double coulomb_k;      /* 0 disables Coulomb */
    double cutoff;         /* force cutoff r_c */
    double skin;           /* neighbour list radius = cutoff + skin */
    double dt;             /* stepwidth */
    double box_lo[3];      /* reflecting walls (boundary_reflect!, Simulator.jl:81-111) */
    double box_hi[3];
    int32_t atomsperleaf;  /* leaf size of the tree used for the neighbour list (divides 32) */
    int32_t rebuild_every; /* steps between neighbour-list rebuilds */
    int32_t order;         /* ND_ORDER_* used for the rebuilds */
    int32_t max_neighbors; /* per-atom list capacity, 0 = sized from the first build */
    int32_t resort_every;  /* every k-th rebuild re-sorts the atoms, the others refit the
                              kept tree; 0 = 1 (always re-sort) */
    int32_t stage_policy;  /* shared-memory staging of a block's neighbour records:
                              0 = sized near the mean union, 1 = the largest union */
    int32_t union_search;  /* how a block of 256 atoms finds the leaves near it (the same
                              leaves either way): ND_UNION_BLOCKS = boxes of the blocks of
                              the kept order, ND_UNION_TREE = breadth-first walk of the
                              LBVH built (re-sort) or refitted (refit) at every rebuild */
    int32_t refit_check_every; /* steps between the early-refit checks inside a window (0 = 1):
                              after every k-th step the engine refits if some atom could pass
                              skin/2 from its list-build position within the next k steps
                              (assuming no step moves an atom more than twice as far as the
                              step before the check) */
    int32_t threads_per_atom; /* threads sharing one atom's neighbour list in the step
                              kernel: 1, 2 or 4; 0 = 4 for a single system whose blocks of
                              256 atoms are fewer than two per SM, else 1 (ensembles: 1) */
    int32_t cta_split;     /* thread blocks of the step kernel per block of 256 atoms with
                              4 threads per atom: 1, 2 or 4 (blocks of 1024, 512 or 256
                              threads, for small systems: more SMs busy); 0 = the most that
                              keep the grid within one thread block per SM; ignored with
                              fewer threads per atom and for ensembles */
} nd_md_params;

#define ND_UNION_BLOCKS 0
#define ND_UNION_TREE   1

/* One system of a batched ensemble: its atom count (a multiple of atomsperleaf),
 * Lennard-Jones parameters and reflecting walls.  Systems never interact. */
typedef struct {
    int32_t n_atoms;
    int32_t reserved;
    double sigma;
    double epsilon;
    double box_lo[3];
    double box_hi[3];
} nd_system;

/* ----------------------------------------------------------------- context */

/* Create a context on CUDA device `device`; allocates its stream and error word. */
nd_status nd_ctx_create(nd_ctx** out, int32_t device);
nd_status nd_ctx_destroy(nd_ctx* ctx);
/* Human-readable text of the last failure on this context (never NULL). */
const char* nd_last_error(const nd_ctx* ctx);
const char* nd_status_string(nd_status st);
/* The context's cudaStream_t, for callers that enqueue their own work. */
void* nd_ctx_stream(nd_ctx* ctx);
nd_status nd_ctx_synchronize(nd_ctx* ctx);
/* The context's device as "<name> sm_<major><minor> x<SMs>" (NUL-terminated,
 * at most len bytes): a key for tuned settings.  No counterpart in the
 * reference. */
nd_status nd_ctx_device_name(const nd_ctx* ctx, char* buf, int32_t len);
/* Number of kernels this library has launched on the context (diagnostics). */
int64_t nd_ctx_launch_count(const nd_ctx* ctx);

/* ------------------------------------------------------------ neighbour search */

/* SpheresBVHSpecs(; neighbor_distance, atom_count, floattype=Float32, atomsperleaf)
 * (BVHTraverse.jl:71-94): ND_ERR_SPEC unless apl divides N and N/apl >= 2. */
nd_status nd_bvh_spec_init(nd_bvh_spec* out, float neighbor_distance, int32_t atom_count,
                           int32_t atomsperleaf);

/* mortoncodes! (BVHTraverse.jl:237-288) on the device: codes[i] for positions
 * xyz (N x 3 Float32).  order selects the reference code or the spatial code. */
nd_status nd_morton_codes_dev(nd_ctx* ctx, const float* xyz, int32_t n, int32_t order,
                              int32_t* codes);

/* Stable ascending sortperm (BVHTraverse.jl:570-573) of non-negative 30-bit
 * codes on the device: codes are sorted in place and perm (0-based) returned. */
nd_status nd_sortperm_dev(nd_ctx* ctx, int32_t* codes, int32_t n, int32_t* perm);

/*
 * leafTreeData(position, spec) (BVHTraverse.jl:544-597) when boxes == ND_BOX_LEAF,
 * TreeData(position, spec) (BVHTraverse.jl:500-543) when boxes == ND_BOX_ATOM.
 * Outputs (each may be NULL): keys (nkeys entries; N-1 for ND_BOX_LEAF, 2nL-1
 * for ND_BOX_ATOM -- extra entries are zero), the sorted APointPrimitive fields
 * index (1-based), morton_code and position (N x 3), and perm (1-based
 * sortperm, the `mortsort` of the reference).  The root box is overwritten with
 * [0,1]^3 as bounding_volume_hierarchy! does (BVHTraverse.jl:856-858).
 * ND_BOX_LEAF with atomsperleaf == 1 returns ND_ERR_SPEC (the reference indexes
 * past its N-1 key array there).
 */
nd_status nd_tree(nd_ctx* ctx, const float* xyz, const nd_bvh_spec* spec, int32_t order,
                  int32_t boxes, nd_gridkey* keys, int64_t nkeys, int32_t* index,
                  int32_t* morton_code, float* position, int32_t* perm);

/*
 * leafbuild_traverse_bvh(position, spec) (BVHTraverse.jl:1423-1428) =
 * leafTreeData + leafneighbor_traverse (:1236-1323); also the pair list of
 * gpubvh_neighborlist (ext/NaiveKA.jl:470-558).  Writes the half pair list
 * (i, j, d) -- every unordered pair with d^2 < r^2 once -- into pi/pj/pd.
 * *count receives the number of pairs; if it exceeds capacity nothing is written
 * and ND_NEED_REALLOC is returned (call again with capacity >= *count, or with
 * capacity 0 to only count).  mode: ND_PAIRS_ORDERED (the order the reference
 * emits on one thread) or ND_PAIRS_UNORDERED (the same pairs in the order the
 * GPU produces them: the two-phase warp-cooperative emission, which needs
 * atomsperleaf == 4; with any other leaf width an unordered request is served
 * by the ordered emission).
 */
nd_status nd_leaf_pairs(nd_ctx* ctx, const float* xyz, const nd_bvh_spec* spec, int32_t order,
                        int32_t mode, int32_t* pi, int32_t* pj, float* pd, int64_t capacity,
                        int64_t* count);

/* Same, device pointers, enqueued on the context stream; *count is a host
 * pointer and the call synchronises once to read it. */
nd_status nd_leaf_pairs_dev(nd_ctx* ctx, const float* xyz, const nd_bvh_spec* spec,
                            int32_t order, int32_t mode, int32_t* pi, int32_t* pj, float* pd,
                            int64_t capacity, int64_t* count);

/*
 * simdbuild_traverse_bvh(position, spec) (ext/NaiveSIMD.jl:706-710) =
 * simdTreeData (:424-480, the leafTreeData tree; atomsperleaf must be 4, else
 * ND_ERR_SPEC) + simdneighbor_traverse (:610-704): the traversal and emission
 * order of leafneighbor_traverse with the SIMD twin's criterion sqrt(d^2) < r
 * (:529,589; the pairs on the boundary can differ from d^2 < r^2).  The
 * reference splits query leaves over threads; ND_PAIRS_ORDERED is its order on
 * one thread.  Same buffer protocol as nd_leaf_pairs.
 */
nd_status nd_simd_leaf_pairs(nd_ctx* ctx, const float* xyz, const nd_bvh_spec* spec,
                             int32_t order, int32_t mode, int32_t* pi, int32_t* pj, float* pd,
                             int64_t capacity, int64_t* count);

/*
 * build_traverse_bvh(position, spec) (BVHTraverse.jl:1416-1421) = TreeData +
 * neighbor_traverse (:1125-1183), the per-atom traversal (and the per-atom
 * kernel gpuneighbor_traverse!, ext/NaiveKA.jl:352-453).  The reference's
 * neighbor_traverse indexes APointPrimitive values that define no getindex at
 * HEAD; this is the traversal it describes: queries 1..N-1 in sorted order
 * start at their own leaf, strict point-in-box tests against +/- r leaf boxes,
 * emit subjects later in sorted order with d^2 < r^2.  Same buffer protocol as
 * nd_leaf_pairs.
 */
nd_status nd_atom_pairs(nd_ctx* ctx, const float* xyz, const nd_bvh_spec* spec, int32_t order,
                        int32_t* pi, int32_t* pj, float* pd, int64_t capacity, int64_t* count);

/*
 * gpubvh_neighborlist!(neighborlist, treedata, spec, backend) (ext/NaiveKA.jl:
 * 597-636; declared at src/PkgExtensions.jl:67): the pair list of new
 * positions from a kept tree.  index and morton_code are the kept treedata's
 * mortonpositions (1-based original index and code of each sorted slot, as
 * nd_tree returns them); xyz holds the new positions in the caller's order.
 * The order and the sorted codes are reused, so the build reproduces the kept
 * topology with the boxes of the new positions -- the refit that TreeData!
 * (BVHTraverse.jl:601-655) intends between rebuilds -- and the pairs are
 * leafneighbor_traverse's over that tree: the pair set equals a fresh build's
 * (every box is exact), the ordered emission follows the kept tree.  keys
 * (nkeys GridKeys, the leafTreeData layout, root box overwritten) and
 * position (N x 3, kept order) receive the refreshed treedata (either may be
 * NULL).  Same pair buffer protocol and modes as nd_leaf_pairs.  ND_ERR_ARG
 * when index is not a permutation of 1..N or morton_code is not ascending.
 * The reference's body reads an undefined `position` at HEAD; the new
 * positions are this call's xyz.
 */
nd_status nd_leaf_pairs_refresh(nd_ctx* ctx, const float* xyz, const nd_bvh_spec* spec,
                                const int32_t* index, const int32_t* morton_code, int32_t mode,
                                nd_gridkey* keys, int64_t nkeys, float* position, int32_t* pi,
                                int32_t* pj, float* pd, int64_t capacity, int64_t* count);

/*
 * The leaf pair-list pipeline of nd_leaf_pairs_dev for callers that cannot
 * allocate device memory (the same kernels: in ND_PAIRS_ORDERED mode the same
 * list bit for bit; in ND_PAIRS_UNORDERED mode with atomsperleaf == 4 a
 * one-pass emission that gives the same pairs with the same distance bits in
 * another order): code running
 * under a host runtime that owns the device memory budget through its own pool,
 * or a time-critical loop in which cudaMalloc/cudaFree would stall the device.
 * No counterpart in the reference (it allocates freely).  Takes no context:
 * positions (xyz, N x 3 Float32) and outputs (pi, pj, pd) are device pointers
 * on the current device; *count is a host pointer; work is enqueued on `stream`
 * (a cudaStream_t, NULL = default stream) and the call synchronises it to read
 * the pair count.  Scratch is one file-scope device array of ~5.3 MB reserved
 * on every GPU that loads the library until the process exits; nothing is
 * allocated.  Limits: atom_count <= 65536 and atomsperleaf >= 2 (in both
 * modes; an unordered request with another leaf width than 4 is served by the
 * ordered emission), otherwise ND_ERR_ARG.  All calls share that array, so
 * calls that overlap on the GPU (other streams or host threads) race:
 * serialise them.  The first call on a device looks up the array's address
 * (with that device current) and keeps it for the life of the process; make
 * that first call before any stream capture.  The kept address does not
 * survive cudaDeviceReset: do not call this entry point after resetting the
 * device in the same process.  Errors are returned as status codes only.
 */
nd_status nd_leaf_pairs_noalloc_dev(const float* xyz, const nd_bvh_spec* spec, int32_t order,
                                    int32_t mode, int32_t* pi, int32_t* pj, float* pd,
                                    int64_t capacity, int64_t* count, void* stream);

/* Order-free 128-bit hash of canonical (min(i,j), max(i,j), bits(d)) triples of
 * a device pair list (for verifying lists too large to copy to the host). */
nd_status nd_pair_hash_dev(nd_ctx* ctx, const int32_t* pi, const int32_t* pj, const float* pd,
                           int64_t npairs, uint64_t hash[2]);

/* ------------------------------------------------------------------ forces */

/*
 * force_lennardjones!(force, pairslist, position) (Forces.jl:15-45) +
 * force_coulomb!(force, pairslist, charge) (Forces.jl:56-66) + sum_forces!
 * (Forces.jl:68-75), fused, with the intended physics: for every listed pair
 * (1-based i, j) with r < cutoff,
 *   F_ij = [24 eps/r^2 (2 (sigma/r)^12 - (sigma/r)^6) + k q_i q_j / r^3] r_ij,
 *   F_i += F_ij, F_j -= F_ij,  U += 4 eps((sigma/r)^12 - (sigma/r)^6) + k q_i q_j / r.
 * x: N x 3 FP64 positions, q: N charges (NULL = no Coulomb), force: N x 3 FP32
 * out (zeroed first), energy: FP64 out (NULL to skip).  The distances in the
 * list are not used; directions need positions.
 */
nd_status nd_forces_pairs(nd_ctx* ctx, const nd_md_params* p, int32_t n, const double* x,
                          const double* q, const int32_t* pi, const int32_t* pj, int64_t npairs,
                          float* force, double* energy);

/*
 * Bug-compatible force calls: what src/Forces.jl computes at HEAD, for scripts
 * that depend on it (the calls above compute the intended physics).  pi, pj, pd:
 * the pair list (1-based indices, Float32 distances) in the order the caller
 * passes it -- the results depend on it; force: N x 3 Float32 out, zeroed
 * first, the three components of an atom always equal.
 *   force_lennardjones!(force, pairslist, position) (Forces.jl:6-45): for each
 *     pair, force[i] .+= (24 eps / d) ((2 sigma / d)^12 - (sigma / d)^6) with
 *     the hard-coded eps = -1f10 and sigma = 0.0001, nothing on force[j];
 *   force_coulomb!(force, pairslist, charge) (Forces.jl:46-66): for each pair,
 *     force[i] .+= q_i q_j / d^2, then force[j] .-= force[i] (the running
 *     total), an order-dependent recurrence run on one GPU thread.
 * Arithmetic follows Julia's promotion of the reference's types (Float32
 * accumulators, distances and charges; Float64 sigma powers).
 */
nd_status nd_compat_force_lennardjones(nd_ctx* ctx, int32_t n, const int32_t* pi,
                                       const int32_t* pj, const float* pd, int64_t npairs,
                                       float* force);
nd_status nd_compat_force_coulomb(nd_ctx* ctx, int32_t n, const int32_t* pi, const int32_t* pj,
                                  const float* pd, int64_t npairs, const float* charge,
                                  float* force);

/*
 * simulate!(sys, spec, clct) as written (src/Simulator.jl:154-256) for a
 * GenericObjectCollection{Float32}, a GenericRandomCollector{Float32} and a
 * SimSpec{Int64, Float32} (integer stepwidth: every operation stays in
 * Float32).  Each step, over the all-pairs list of unique_pairs
 * (src/Neighbors/AllToAll.jl:65-80, distances from the previous step):
 *   F    = force_lennardjones!(threshold_pairs(list, 0.01)) + force_coulomb!(list)
 *   x   += v dt + (F/m) dt^2 / 2
 *   v   += (F/m + Fnext/m) dt / 2        Fnext: the previous step's all-pairs forces
 *   Fnext = force_lennardjones!(list) + force_coulomb!(list);  boundary_reflect!
 *   update_pairslist!;  every 10th step rescale_velocity!;  log the positions
 * with the compat force formulas above.  position, velocity, force: N x 3
 * Float32, in/out (force in: the first step's Fnext).  mass, charge: N.
 * poslog: NULL or (duration + 1) x N x 3 Float32 out: frame k the positions
 * after step k, frame 0 the final positions (the reference's poslog[1] is
 * sys.position itself).  1 <= n <= 65536 (the list holds n(n-1)/2 pairs).
 * A negative rescale_velocity! radicand (Julia's DomainError) stops the run
 * after that step's pair update with ND_ERR_ARG; the state is then the one
 * the reference holds when it throws.
 */
typedef struct nd_compat_sim {
    float min_dim[3];          /* GenericRandomCollector minDim */
    float max_dim[3];          /* GenericRandomCollector maxDim */
    float temperature;         /* GenericRandomCollector temperature (Tf) */
    int64_t objectnumber;      /* GenericRandomCollector objectnumber */
    int64_t stepwidth;         /* SimSpec stepwidth (Int64) */
    int64_t duration;          /* SimSpec duration (steps) */
    float velocity_dampening;  /* SimSpec velocityDampening (gamma) */
} nd_compat_sim;

nd_status nd_compat_simulate(nd_ctx* ctx, const nd_compat_sim* spec, int32_t n, float* position,
                             float* velocity, float* force, const float* mass,
                             const float* charge, float* poslog);

/*
 * collect_objects(clct::GenericRandomCollector) (src/MDInput.jl:305-369) on
 * the device: masses, charges and positions uniform in the collector's
 * ranges (generate_positions, :175-190), velocities T * veldist * 3N kb / m
 * per component with veldist a Float32 uniform split normalised to sum 1
 * (randomvelocity) or T / N * 3N kb / m, and unique_pairs_prune (:228-259) as
 * written: atom i (1-based, i <= N - 2) with an atom j in i+1 .. N-1 closer
 * than minimumdistance gets Inf coordinates (the reference's re-placement
 * loop never runs: its condition tooClose < 0 is never true); *pruned (may
 * be NULL) receives their number.  Draws come from a counter-based splitmix64
 * stream of `seed` instead of Julia's global RNG, so values match the
 * reference's distributions, not its draws.  position, velocity: N x 3
 * Float32 out; mass, charge: N Float32 out; N = objectnumber <= 2^20 (the
 * pruning compares all pairs, as the reference does).
 */
typedef struct nd_collector {
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
} nd_collector;

nd_status nd_collect_objects(nd_ctx* ctx, const nd_collector* collector, uint64_t seed,
                             float* position, float* velocity, float* mass, float* charge,
                             int64_t* pruned);

/*
 * Forces and energy of a configuration with the library's own neighbour search
 * (spatial-order leaf BVH at radius p->cutoff): the fused hot-path force kernel
 * run once.  Same physics and outputs as nd_forces_pairs.
 */
nd_status nd_forces(nd_ctx* ctx, const nd_md_params* p, int32_t n, const double* x,
                    const double* q, float* force, double* energy);

/* ---------------------------------------------------------------- dynamics */

/*
 * Device-resident simulation (the GPU form of simulate!, Simulator.jl:154-256,
 * with kick-drift-kick velocity Verlet):
 *   v += dt/2 F/m;  x += dt v;  boundary_reflect!;  [rebuild every R steps];
 *   F = F(x);  v += dt/2 F/m.
 * x, v: N x 3 FP64 host arrays; q (charges) and m (masses) may be NULL (q = 0
 * disables Coulomb, m = 1).  The state is copied to the device once.
 */
nd_status nd_md_create(nd_ctx* ctx, const nd_md_params* p, int32_t n, const double* x,
                       const double* v, const double* q, const double* m, nd_md** out);
/* Same, from device arrays (x, v: N x 3 FP64; q, m: N FP64 or NULL). */
nd_status nd_md_create_dev(nd_ctx* ctx, const nd_md_params* p, int32_t n, const double* x,
                           const double* v, const double* q, const double* m, nd_md** out);
nd_status nd_md_destroy(nd_md* md);
/* Advance `steps` steps; enqueued on the context stream (captured CUDA graphs of
 * one rebuild window).  Does not synchronise. */
nd_status nd_md_run(nd_md* md, int64_t steps);
/* Synchronise and check the device error word (overflow, non-finite, ...). */
nd_status nd_md_sync(nd_md* md);
/* Copy the state back in the caller's original atom order (each may be NULL):
 * x, v (N x 3 FP64), f (N x 3 FP32 forces at the current positions). */
nd_status nd_md_get(nd_md* md, double* x, double* v, float* f);
/* Same into device buffers. */
nd_status nd_md_get_dev(nd_md* md, double* x, double* v, float* f);
/* Potential and kinetic energy (FP64 reductions) at the current step. */
nd_status nd_md_energy(nd_md* md, double* potential, double* kinetic);
/* Steps taken, rebuilds done, pairs in the current list, list capacity. */
nd_status nd_md_stats(nd_md* md, int64_t* steps, int64_t* rebuilds, int64_t* list_pairs,
                      int32_t* capacity);
/* Engine diagnostics (nd_md_diagnostics). */
typedef struct {
    int64_t skin_violations; /* atom-steps computed with a list from which an atom had
                                moved more than skin/2: the list may then miss pairs (none
                                with a check after every step; with sparser checks, a
                                system moving too fast for them) */
    int32_t max_neighbors;   /* largest per-atom neighbour count of any build */
    int32_t reserved;
    int64_t resorts;         /* window rebuilds that re-sorted the atoms */
    int64_t refits;          /* window rebuilds that refitted the kept tree */
    int64_t early_refits;    /* refits inside a window: at a check that found some atom
                                able to pass skin/2 before the next check */
    int64_t resort_kernels;  /* kernels of one re-sort rebuild */
    int64_t refit_kernels;   /* kernels of one refit */
    int64_t body_kernels;    /* kernels run so far inside captured conditional nodes
                                (not in nd_ctx_launch_count) */
} nd_md_diag;

/* Rebuilds are decided on the device: a window re-sorts every resort_every-th
 * time or when a list has passed 90% of its capacity since the last re-sort,
 * and refits otherwise; a checked step (every refit_check_every-th = k-th step
 * of a window) after which some atom could pass skin/2 from its list-build
 * position before the next check (its displacement plus 2 (k - 1) times its
 * last move, twice it for k = 1, reaches 95% of skin/2) is followed by an
 * early refit. */
nd_status nd_md_diagnostics(nd_md* md, nd_md_diag* out);
/* The engine's current neighbour lists as directed pairs (pi[k], pj[k]) of
 * 1-based caller indices -- every list entry, so each unordered pair appears
 * once from each side -- in no particular order, with near[k] = 1 for entries
 * of the near segment (pairs closer than 1.3 sigma + 0.1 at the list build,
 * whose forces are evaluated with exact r^2 residuals).  With capacity below
 * the entry count, *count receives the count and ND_NEED_REALLOC is returned.
 * Host arrays; synchronises.  No counterpart in the reference, whose pair
 * lists are plain vectors (leafneighbor_traverse, src/Neighbors/
 * BVHTraverse.jl:1236): the engine's lists are read back for verification. */
nd_status nd_md_list_pairs(nd_md* md, int32_t* pi, int32_t* pj, uint8_t* near,
                           int64_t capacity, int64_t* count);
/* Advance `steps` steps without captured graphs, timing each step kernel with
 * its own pair of CUDA events on the context stream: ms[k] (host array of
 * `steps`) receives the k-th step kernel's duration.  Synchronises. */
nd_status nd_md_step_times(nd_md* md, int32_t steps, float* ms);
/*
 * rescale_velocity!(velocity, Tf, gamma, mass, objectcount) (Simulator.jl:119-144),
 * which simulate! applies every 10 steps (Simulator.jl:241-243): after every
 * `every`-th step, on the integer-step velocities,
 *   Ti = sum_i (2 / (3 N kb)) |v_i| m_i / 2   (kb = 1; the reference sums |v|, not v^2),
 *   beta = (1 + gamma (Tf / Ti - 1))^0.5,   v_i *= beta.
 * Ti <= 0 leaves the velocities unchanged; a negative radicand (the
 * reference's DomainError) leaves them unchanged and the next sync returns
 * ND_ERR_ARG.  every = 0 switches it off.  Single-system engines only.
 */
nd_status nd_md_set_thermostat(nd_md* md, double temperature, double gamma, int32_t every);
/*
 * The position log of simulate! (poslog, Simulator.jl:167,245), kept on the
 * device: after every `every`-th step the positions (caller order, N x 3 FP64)
 * go into a ring of `frames` frames.  every = 0 switches it off.  Setting it
 * restarts the frame count.
 */
nd_status nd_md_set_log(nd_md* md, int32_t every, int32_t frames);
/* Frames logged so far (including frames the ring has overwritten). */
nd_status nd_md_log_count(nd_md* md, int64_t* count);
/* Copy frames [first, first + nframes) (frame k = the k-th logged step) to a host
 * array of nframes x N x 3 FP64; frames no longer in the ring are ND_ERR_ARG. */
nd_status nd_md_log_read(nd_md* md, int64_t first, int64_t nframes, double* out);
/* Number of kernel launches one nd_md_run(steps) enqueues (for diagnostics). */
int64_t nd_md_launches_per_run(nd_md* md, int64_t steps);

/*
 * Batched ensemble: `nsys` independent systems advanced together by one engine
 * (each step is one launch over all systems' atoms; rebuild windows are
 * captured CUDA graphs).  x, v: (sum n_atoms) x 3 FP64, systems concatenated
 * in order; q, m may be NULL.  p supplies the shared settings (cutoff, skin,
 * dt, coulomb_k, atomsperleaf, rebuild_every, resort_every, stage_policy);
 * its sigma, epsilon and walls are ignored in favour of each system's.  The
 * result is an nd_md: nd_md_run / get / sync / diagnostics apply unchanged and
 * nd_md_energy returns the ensemble totals.  No counterpart in the reference
 * (it runs one system per simulate! call).
 */
nd_status nd_batch_create(nd_ctx* ctx, const nd_md_params* p, int32_t nsys, const nd_system* sys,
                          const double* x, const double* v, const double* q, const double* m,
                          nd_md** out);
/* Same, from device arrays. */
nd_status nd_batch_create_dev(nd_ctx* ctx, const nd_md_params* p, int32_t nsys,
                              const nd_system* sys, const double* x, const double* v,
                              const double* q, const double* m, nd_md** out);
/* Per-system potential and kinetic energies (arrays of nsys; either may be NULL). */
nd_status nd_batch_energies(nd_md* md, double* potential, double* kinetic);

/*
 * Autotuner: times short runs of candidate engine settings on copies of the
 * given state (host arrays; the state is not advanced) and writes the fastest
 * into *best (skin -- p->skin - 0.2 to p->skin + 0.2 in steps of 0.1, not below
 * 0.1 --, atomsperleaf -- the leaf/traversal width --, resort_every,
 * stage_policy, union_search, refit_check_every -- 1, 2 or 3 -- and, for a
 * plain engine, threads_per_atom -- 1, 2 or 4 -- and cta_split -- 1, 2 or 4 with
 * 4 threads per atom; every other field copied from *p), tuning one setting at
 * a time.  nsys == 0 tunes a plain engine (sys ignored).  Candidates
 * change only the summation order of the forces and the steps at which early
 * refits may run, not which pairs interact.  trial_steps: timed steps per candidate
 * (rounded up to whole rebuild windows).  seconds_per_step (may be NULL)
 * receives the winner's time per MD step.
 */
nd_status nd_md_autotune(nd_ctx* ctx, const nd_md_params* p, int32_t n, int32_t nsys,
                         const nd_system* sys, const double* x, const double* v, const double* q,
                         const double* m, int32_t trial_steps, nd_md_params* best,
                         double* seconds_per_step);

/*
 * simulate!(sys, spec, clct) (Simulator.jl:154-256) with host arrays in and out:
 * x, v (N x 3 FP64) are advanced `steps` steps in place and f (N x 3 FP32,
 * may be NULL) receives the forces at the final positions.
 */
nd_status nd_simulate(nd_ctx* ctx, const nd_md_params* p, int32_t n, double* x, double* v,
                      float* f, const double* q, const double* m, int64_t steps);

/* Diagnostics (nd_md_diag) of the engine that the context's last nd_simulate
 * call ran: a caller checks skin_violations > 0 -- atom-steps computed on a
 * list that an atom had left by more than skin/2, so that pairs may have been
 * missed -- and raises the skin or the check frequency.  ND_ERR_ARG when no
 * call has run.  No counterpart in the reference (it rebuilds its all-pairs
 * list every step and has no skin). */
nd_status nd_simulate_diagnostics(nd_ctx* ctx, nd_md_diag* out);

/* ------------------------------------------------------------------ adjoint */

/*
 * Differentiable trajectory: `steps` kick-drift-kick steps of the engine from
 * (x0, v0), then the Gaussian-smoothed pair-distance histogram of the final
 * positions,
 *   h_b = (1/N) sum_{i<j, r_ij < r_max} s(r_ij) exp(-(r_ij - c_b)^2 / (2 width^2)),
 *   c_b = (b + 1/2) r_max / bins,  s = 1 below r_switch, a C2 switch to 0 at r_max,
 * and the loss L = sum_b (h_b - target_b)^2.  The backward pass is the
 * hand-written adjoint of that program (reverse steps over the same
 * neighbour lists, segments of checkpoint_every steps recomputed from their
 * checkpoints): dL/dx0, dL/dv0, dL/dsigma, dL/depsilon.  Wall clamps and the
 * force cutoff are differentiated as the piecewise program they are.
 * Rebuilds: a re-sort every resort_every windows (0 = 5), refits between, and
 * early refits decided on the device in the forward pass (as nd_md_run does)
 * and replayed from its record in the backward pass.  Results do not depend
 * on checkpoint_every: every interval gives the same bits.  A forward pass in
 * which an atom still moved more than skin/2 from its list-build position
 * returns ND_ERR_OVERFLOW.  No counterpart in the reference (it has no
 * derivative code); the Julia side is a ChainRulesCore.rrule over these calls.
 */
typedef struct nd_adj nd_adj;
typedef struct {
    int32_t steps;            /* K: a multiple of checkpoint_every */
    int32_t checkpoint_every; /* a multiple of resort_every * rebuild_every; 0 = 50 */
    int32_t bins;             /* 1..1024 */
    int32_t reserved;
    double r_max;             /* histogram range [0, r_max], r_max <= cutoff */
    double width;             /* Gaussian width; 0 = r_max / bins */
    double r_switch;          /* start of the pair-weight switch; < 0 = r_max - 0.25 */
} nd_adj_spec;

/* x0, v0: N x 3 FP64 host arrays; q, m: N or NULL.  p as for nd_md_create. */
nd_status nd_adj_create(nd_ctx* ctx, const nd_md_params* p, int32_t n, const double* x0,
                        const double* v0, const double* q, const double* m,
                        const nd_adj_spec* spec, nd_adj** out);
nd_status nd_adj_destroy(nd_adj* adj);
/* Lennard-Jones parameters of later passes. */
nd_status nd_adj_set_params(nd_adj* adj, double sigma, double epsilon);
/* Target histogram (bins values, host; NULL = zeros). */
nd_status nd_adj_set_target(nd_adj* adj, const double* target);
/* Forward pass: hist (bins) and loss out (either may be NULL). */
nd_status nd_adj_forward(nd_adj* adj, double* hist, double* loss);
/* Backward pass after a forward pass: dL/dx0, dL/dv0 (N x 3, caller order),
 * dL/dsigma, dL/depsilon (each may be NULL). */
nd_status nd_adj_backward(nd_adj* adj, double* dx0, double* dv0, double* dsigma,
                          double* depsilon);
/* Final positions x_K (N x 3, caller order) of the last forward pass. */
nd_status nd_adj_final(nd_adj* adj, double* x);
/* Device durations (CUDA events on the context stream) of the last forward
 * and backward passes, in ms (either may be NULL; -1 for a pass not run yet). */
nd_status nd_adj_times(nd_adj* adj, float* forward_ms, float* backward_ms);

/* ------------------------------------------------------------ synthetic inputs */

/* Seeded host-side generators for benchmark and test inputs (splitmix64). */
/* Uniform Float32 positions in [lo, lo + side)^3. */
nd_status nd_synth_uniform(uint64_t seed, int32_t n, double lo, double side, float* xyz);
/* Uniform positions in [0, side)^3 with no two atoms closer than dmin (random
 * sequential addition; MDInput.jl's GenericRandomCollector.minimumdistance). */
nd_status nd_synth_uniform_mindist(uint64_t seed, int32_t n, double side, double dmin,
                                   double* xyz);
/* nclusters isotropic Gaussian clusters of n/nclusters points, centres uniform in
 * [0, side)^3, per-cluster sigma uniform in [smin, smax]. */
nd_status nd_synth_clusters(uint64_t seed, int32_t n, int32_t nclusters, double side,
                            double smin, double smax, float* xyz);
/* N(0, s^2) per component. */
nd_status nd_synth_normal(uint64_t seed, int64_t count, double s, double* out);
/* +/-1 charges, exactly half each, random assignment (n even). */
nd_status nd_synth_charges(uint64_t seed, int32_t n, double* q);

#ifdef __cplusplus
}
#endif
#endif
