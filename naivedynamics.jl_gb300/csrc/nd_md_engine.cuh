// nd_md_engine.cuh -- internal interface of the device-resident MD engine
// (nd_md.cu) for the kernels built on its state and neighbour lists
// (nd_adjoint.cu): layouts, the engine object and its building blocks.
#pragma once

#include "nd_internal.cuh"

namespace nd {

constexpr int kBlock = 256;          // atoms per block in the list and step kernels

// Fixed-point frame of the pair records: x_fp = rint((x - origin) * scale).
struct Frame {
    double o[3];
    double s;
};

struct SetPtrs {
    double* x[3];
    double* w[3];
    double* q;
    double* im;
    int32_t* orig;
    int32_t* sid;  // batched ensembles: system of each atom (nullptr for one system)
};

// Per-system constants of a batched ensemble.  Each system keeps its own
// fixed-point frame (origin o, scale s) and is placed in its own slot of the
// tree frame (Float32 positions = x + off), slots far enough apart that no
// neighbour-list pair crosses systems.  Pair constants are in the system's
// fixed-point units.
struct SysRow {
    double o[3];                 // fixed-point frame origin
    double os[3];                // o * s
    double off[3];               // tree-frame offset
    double lo[3], hi[3];         // walls
    double s;                    // fixed-point scale
    int32_t lo_fp[3], hi_fp[3];  // walls in fixed point
    float sig2u, eps24u, eps4, rc2u, kcu, kceu, hs2u, hsu;
};

__device__ __forceinline__ int32_t to_fixed(double x, double o, double s, int32_t* err,
                                            int32_t who) {
    double t = fma(x, s, -(o * s));
    if (!(t > -2147483000.0 && t < 2147483000.0)) {
        set_error(err, isfinite(x) ? ND_ERR_RANGE : ND_ERR_NONFINITE, who);
        t = 0.0;
    }
    return __double2int_rn(t);
}

struct StepArgs {
    int32_t n, apl, ucap, lcap;
    int32_t smrec;  // union records staged in shared memory (the rest read from global)
    const int32_t* __restrict__ ulist;
    const int32_t* __restrict__ ucount;
    const uint16_t* __restrict__ llist;
    const int32_t* __restrict__ ncount;
    const int4* __restrict__ rec_in;
    int4* __restrict__ rec_out;
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
    double os[3];       // origin * scale (fixed-point offset)
    int32_t lo_fp[3], hi_fp[3];  // walls in fixed point (filter for the exact FP64 test)
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
    DevBuf set_buf[2], rec_buf[2], recb, xyz32, pos32, keys, store, bbox, ulist, ucount, llist_leaf,
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
// of kBlock atoms, slot-major: entry s of the block's thread t is element
// s * kBlock + t, so a warp reading its atoms' s-th entries reads 64
// contiguous bytes.
__device__ __forceinline__ int64_t llist_at(int32_t s, int32_t t) {
    return (int64_t)s * kBlock + t;
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
