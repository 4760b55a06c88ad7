// nd_md_engine.cuh -- internal interface of the device-resident MD engine
// (nd_md.cu) for the kernels built on its state and neighbour lists
// (nd_adjoint.cu): layouts, the engine object and its building blocks.
#pragma once

#include "nd_internal.cuh"

namespace nd {

constexpr int kBlock = 256;          // atoms per block in the list and step kernels

// Fixed-point frame of the pair records: x_fp = rint((x - origin) * scale)
// modulo 2^32.  The scale is the largest power of two at which every listed
// pair's per-axis separation stays below 2^31 grid units, so the wrapped
// int32 difference of two records is the exact separation even where the
// records themselves wrap.  lim bounds |x_fp| before the wrap: positions
// beyond the walls by more than the frame's margin are range errors.
struct Frame {
    double o[3];
    double s;
    double lim;
};

struct SetPtrs {
    double* x[3];
    double* w[3];
    double* q;
    double* im;
    int32_t* orig;
    int32_t* sid;  // batched ensembles: system of each atom (nullptr for one system)
};

// Near pairs (separation below 1.3 sigma when evaluated) carry most of the
// rounding error of single-precision pair terms: the force of a pair near the
// potential minimum is a difference of two nearly equal terms, so a relative
// error in r^2 reaches the force amplified about 30-fold.  Their terms are
// evaluated in two-float arithmetic (see accum_near in nd_md.cu).  The list
// build puts pairs closer than rnb (1.3 sigma + 0.1) in a separate segment of
// each atom's list; a pair of the other segment that comes closer than 1.3
// sigma during the window is caught by the rn2u test.
struct NearK {
    float rn2u;     // (1.3 sigma S)^2: evaluate accurately below this
    float sig2lo;   // sigma^2 S^2 - sig2u (rounding of the LJ constant)
    float e24lo;    // 24 eps S - eps24u
    float kclo;     // k S^2 - kcu
    float rc2lo;    // (r_c S)^2 - rc2u: the cutoff as a two-float value
    float rnb2;     // (1.3 sigma + 0.1)^2 in physical units: list segment bound
    int32_t hmask;  // clears the low k bits of a separation: the exact split
};

// Pair records hold the position on the grid of scale S (coarse, int32 modulo
// 2^32); a second record per atom holds the next 16 bits of each coordinate
// (the fine grid, scale S * 2^16), which only the near-pair terms read:
// coarse = floor(X / 2^16) and fine = X mod 2^16 for X = rint((x - o) S 2^16).
constexpr double kFine = 65536.0;

// Per-system constants of a batched ensemble.  Each system keeps its own
// fixed-point frame (origin o, scale s) and is placed in its own slot of the
// tree frame (Float32 positions = x + off), slots far enough apart that no
// neighbour-list pair crosses systems.  Pair constants are in the system's
// fixed-point units.
struct SysRow {
    double o[3];                 // fixed-point frame origin
    double os[3];                // o * s * 2^16
    double off[3];               // tree-frame offset
    double lo[3], hi[3];         // walls
    double s;                    // fixed-point scale (coarse grid)
    double lim;                  // range bound of x_fp before the wrap (coarse units)
    int64_t lo_fp[3], hi_fp[3];  // walls on the fine grid (before the wrap)
    float sig2u, eps24u, eps4, rc2u, kcu, kceu, hs2u, hsu;
    NearK nk;                    // near-pair constants
};

// Records keep x_fp modulo 2^32; the difference of two records, taken modulo
// 2^32, is the exact separation of any listed pair.
__device__ __forceinline__ int32_t idiff(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a - (uint32_t)b);
}

// Coarse record coordinate (modulo 2^32) and its fine bits of position x.
__device__ __forceinline__ int32_t to_fixed(double x, double o, double s, double lim,
                                            int32_t* err, int32_t who, uint32_t& fine) {
    const double sf = s * kFine;
    double t = fma(x, sf, -(o * sf));
    if (!(t > -lim * kFine && t < lim * kFine)) {
        set_error(err, isfinite(x) ? ND_ERR_RANGE : ND_ERR_NONFINITE, who);
        t = 0.0;
    }
    const long long X = __double2ll_rn(t);
    fine = (uint32_t)X & 0xffffu;
    return (int32_t)(uint32_t)(unsigned long long)(X >> 16);
}
__device__ __forceinline__ uint2 pack_fine(uint32_t fx, uint32_t fy, uint32_t fz) {
    return make_uint2(fx | (fy << 16), fz);
}

struct StepArgs {
    int32_t n, apl, ucap, lcap;
    int32_t first;     // the first step after an upload (a half kick only)
    int32_t has_mass;  // im holds inverse masses (else all masses are 1)
    int32_t smrec;  // union records staged in shared memory (the rest read from global)
    const int32_t* __restrict__ ulist;
    const int32_t* __restrict__ ucount;
    const uint16_t* __restrict__ llist;
    const int32_t* __restrict__ ncount;
    const int4* __restrict__ rec_in;
    int4* __restrict__ rec_out;
    const uint2* __restrict__ recf_in;  // fine bits of the records
    uint2* __restrict__ recf_out;
    double* x[3];
    double* w[3];
    const double* __restrict__ im;
    float4* __restrict__ f_out;
    double* __restrict__ v_out[3];  // measure mode: integer-step velocity
    double* __restrict__ acc;       // measure mode: [0] potential, [1] kinetic
    const int4* __restrict__ rec_build;     // records at the last rebuild
    unsigned long long* __restrict__ diag;  // [0] atom-steps moved > skin/2 since the build
    int32_t* err;
    float half_skin2u;  // (skin/2)^2 in fixed-point units
    double os[3];       // origin * scale * 2^16 (fixed-point offset, fine grid)
    int64_t lo_fp[3], hi_fp[3];  // walls on the fine grid (filter for the exact FP64 test)
    NearK nk;           // near-pair constants (one system)
    // pair constants in fixed-point units (S = frame scale)
    float rc2u;    // (r_c S)^2
    float sig2u;   // (sigma S)^2
    float eps24u;  // 24 eps S
    float eps4;    // 4 eps
    float kcu;     // k S^2   (Coulomb force)
    float kceu;    // k S     (Coulomb energy)
    float hdt;     // dt / 2
    double dt;
    double lo[3], hi[3];
    Frame fr;
    const int32_t* __restrict__ sid;  // batched ensembles: system of each sorted atom
    const SysRow* __restrict__ sys;   // and the per-system constants
    int32_t nsys;
    // early refit: ctl[0] request flag, ctl[1] finished-block tickets; inside a
    // captured window the last block sets `cond` for the conditional refit node
    float hsu;  // skin/2 in fixed-point units (early-refit trigger)
    unsigned* ctl;
    cudaGraphConditionalHandle cond;
    int32_t use_cond;
    // this step votes for an early refit (a check follows it); the vote
    // covers the next trig_k / 2 + 1 steps
    int32_t vote;
    float trig_k;
    // the next step uses this step's list unchecked: an atom past skin/2 is a
    // skin violation
    int32_t unchecked;
};

struct MDEngine {
    Ctx* parent = nullptr;
    Ctx sub;  // private scratch for the rebuild pipeline (stable pointers for graphs)
    nd_md_params p{};
    int32_t n = 0, nL = 0, apl = 4, nblocks = 0;
    int32_t lcap = 0, ucap = 0, upow2 = 0, fcap = 0, lcap_leaf = 0, ucap_sm = 0;
    bool has_q = false, has_m = false;
    bool first = true;
    int cur = 0;            // current state set
    int rc = 0;             // current record buffer
    int32_t in_window = 0;  // steps done in the current window
    bool rebuild_due = false;
    int64_t steps = 0, rebuilds = 0;
    Frame fr{};
    DevBuf set_buf[2], rec_buf[2], recf_buf[2], recb, xyz32, pos32, keys, store, bbox, ulist, ucount, llist_leaf,
        lcount_leaf, llist, ncount, f, vtmp, acc, aos, diag, sysrow, sid_in;
    // batched ensemble (nsys > 0): per-system rows and the Hilbert grid whose
    // level-log2(G) cells are the systems' slots
    int32_t nsys = 0;
    float tree_frame[6] = {0, 0, 0, 0, 0, 0};
    // early refits: ctl = {request flag, block tickets, early refits done};
    // the first window after an upload is captured too (graph_first), and the
    // conditional refit bodies are captured on cap_stream
    DevBuf ctl;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph_first = nullptr;
    int64_t graph_first_launches = 0, refit_kernels = 0;
    SetPtrs set[2];
    // one captured window: a device-decided rebuild (re-sort or refit) and R
    // steps with conditional early refits; the live state is always set 0
    cudaGraphExec_t graph_main = nullptr;
    int32_t resort_every = 1;  // re-sort (new order + topology) every k-th window, refit between
    int32_t check_every = 1;   // steps between early-refit checks
    int64_t graph_main_launches = 0;  // kernel nodes of the window graph outside conditional bodies
    int64_t resort_kernels = 0;       // kernels of one re-sort rebuild
    int64_t eager_bodies = 0;         // kernels of rebuild bodies run eagerly (counted by the host)
    size_t step_smem = 0, union_smem = 0, lists_smem = 0;
    int32_t lists_smpos = 0;  // positions the list kernel stages in shared memory
    int32_t split = 1;  // thread blocks of the step kernel per block of kBlock atoms
    int32_t tpa = 1;  // threads per atom of the step kernel
    // observers of the step loop: thermostat (rescale_velocity!) and position log
    double thermo_T = 0.0, thermo_gamma = 0.0;
    int32_t thermo_every = 0, log_every = 0;
    int64_t log_frames = 0;
    DevBuf obs, obs_part, logbuf;  // obs: frames logged, thermostat runs, last beta
    int64_t thermo_kernels = 0, log_kernels = 0;
};

enum { RB_RESORT = 0, RB_REFIT = 1 };

// Per-atom neighbour lists (uint16 indices into the block's union), per block
// of kBlock atoms, slot-major: slot s of the block's thread t is element
// s * kBlock + t, so a warp reading its atoms' s-th entries reads 64
// contiguous bytes.  Each list has two segments: the near entries from slot
// 0 upwards and the others from slot lcap - 1 downwards; ncount packs the
// two counts (near in the low 16 bits).
__device__ __forceinline__ int64_t llist_at(int32_t s, int32_t t) {
    return (int64_t)s * kBlock + t;
}
__device__ __forceinline__ int32_t list_near(int32_t c) { return c & 0xffff; }
__device__ __forceinline__ int32_t list_total(int32_t c) { return (c & 0xffff) + (c >> 16); }
// slot of logical entry s (near entries first, then the others in build order)
__device__ __forceinline__ int32_t list_slot(int32_t s, int32_t c, int32_t lcap) {
    const int32_t nn = c & 0xffff;
    return s < nn ? s : lcap - 1 - (s - nn);
}

// Rebuild of the neighbour lists (re-sort or refit; see nd_md.cu).
nd_status md_rebuild(MDEngine* m, int kind, int rec = -1, unsigned* counter = nullptr,
                     bool sizing = false);
// Step-kernel arguments for the current state set, reading records `rec_in`.
StepArgs md_step_args(MDEngine* m, int rec_in);
// One velocity-Verlet step kernel (force, kick, drift, walls, next record).
void md_launch_step(MDEngine* m, const StepArgs& a, bool first);
// Copy x, v, q, m into state set 0 in the caller's order (host or device).
nd_status md_upload(MDEngine* m, const double* xd, const double* vd, const double* qd,
                    const double* md_, bool host);

// Conditional node after the work captured so far on c->stream.  nbody = 1:
// IF (body 0 runs when the condition is non-zero); nbody = 2: IF/ELSE (body 1
// runs when it is zero).  Each body is captured on cap_stream by body(k); its
// kernels are counted apart (they run only when chosen) into nk_out[k] when
// nk_out is given.
template <class F>
inline nd_status md_add_cond_node(MDEngine* m, cudaGraphConditionalHandle h, int nbody,
                                  F&& body, int64_t* nk_out = nullptr) {
    Ctx* c = &m->sub;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, &deps, nullptr, &nd);
    if (e != cudaSuccess) return cuda_fail(c, e, "capture info");
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = (unsigned)nbody;
    cudaGraphNode_t node = nullptr;
    e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &np);
    if (e != cudaSuccess) return cuda_fail(c, e, "conditional node");
    nd_status st = ND_OK;
    cudaStream_t main = c->stream;
    for (int k = 0; k < nbody && st == ND_OK; ++k) {
        c->stream = m->cap_stream;
        e = cudaStreamBeginCaptureToGraph(m->cap_stream, np.conditional.phGraph_out[k], nullptr,
                                          nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) { st = cuda_fail(c, e, "body capture"); break; }
        const int64_t l0 = c->launches;
        st = body(k);
        const int64_t nk = c->launches - l0;
        c->launches = l0;
        cudaGraph_t out = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(m->cap_stream, &out);
        if (e2 != cudaSuccess && st == ND_OK) st = cuda_fail(c, e2, "body capture");
        if (st == ND_OK && nk_out) nk_out[k] = nk;
    }
    c->stream = main;
    if (st) return st;
    e = cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1,
                                            cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return cuda_fail(c, e, "capture dependencies");
    return ND_OK;
}

// A conditional handle of the graph being captured on the engine stream; its
// value resets to 0 at every launch and the kernel before its node sets it.
inline nd_status md_cond_handle(MDEngine* m, cudaGraphConditionalHandle* h) {
    Ctx* c = &m->sub;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, nullptr, nullptr, nullptr);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(h, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return cuda_fail(c, e, "conditional handle");
    return ND_OK;
}

}  // namespace nd
