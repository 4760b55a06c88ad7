// nd_internal.cuh -- shared device helpers and the internal C++ interface between
// the kernel translation units (nd_bvh.cu, nd_md.cu) and the C ABI (nd_capi.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>
#include <string>

#include "../../include/naivegpu.h"
#include <nvtx3/nvToolsExt.h>

namespace nd {

struct MDEngine;

// ------------------------------------------------------------------ errors

// Device error word layout: [0] first error status, [1] its info (an index),
// [2] largest per-atom neighbour count seen (overflow diagnostics), [3] spare.
constexpr int kErrWords = 4;

__device__ __forceinline__ void set_error(int32_t* err, int32_t code, int32_t info) {
    if (atomicCAS(err, 0, code) == 0) atomicExch(err + 1, info);
}

// ------------------------------------------------------- IEEE helpers (Julia)

// Base.min / Base.max on IEEE floats: sign of x - y picks the argument, so -0
// orders below +0.  Inputs are finite here (non-finite positions are rejected).
__device__ __forceinline__ float jl_min(float x, float y) {
    float d = __fsub_rn(x, y);
    return signbit(d) ? x : y;
}
__device__ __forceinline__ float jl_max(float x, float y) {
    float d = __fsub_rn(x, y);
    return signbit(d) ? y : x;
}

// sum((a - b).^2) on SVector{3,Float32}: left-to-right, no contraction.
__device__ __forceinline__ float dist2_ref(float ax, float ay, float az, float bx, float by,
                                           float bz) {
    float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Order-preserving float <-> uint32 map for atomic min/max of floats.
__device__ __forceinline__ uint32_t f2o(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__host__ __device__ inline float o2f(uint32_t o) {
    uint32_t b = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// 3-D Hilbert index of a cell of a 1024^3 grid (10 bits per axis, 30-bit
// result), by J. Skilling's transpose method ("Programming the Hilbert curve",
// AIP Conf. Proc. 707, 2004): undo the excess work per bit plane, Gray-encode,
// then interleave the transposed bits, x first.  Consecutive indices are
// face-adjacent cells, so runs of consecutive atoms stay spatially compact.
__host__ __device__ inline uint32_t hilbert3_10(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t X[3] = {x & 1023u, y & 1023u, z & 1023u};
    for (uint32_t Q = 1u << 9; Q > 1u; Q >>= 1) {
        const uint32_t P = Q - 1u;
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                const uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];
    X[2] ^= X[1];
    uint32_t t = 0;
    for (uint32_t Q = 1u << 9; Q > 1u; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1u;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    uint32_t h = 0;
    for (int q = 9; q >= 0; --q)
        for (int i = 0; i < 3; ++i) h = (h << 1) | ((X[i] >> q) & 1u);
    return h;
}

__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Order-free pair hash contribution of one canonical (min, max, bits(d)) triple.
__host__ __device__ inline void pair_hash_one(int32_t i, int32_t j, float d, uint64_t& h0,
                                              uint64_t& h1) {
    uint32_t a = (uint32_t)(i < j ? i : j);
    uint32_t b = (uint32_t)(i < j ? j : i);
    uint32_t db;
    memcpy(&db, &d, 4);
    uint64_t k = ((uint64_t)a << 32) | (uint64_t)b;
    uint64_t x = mix64(k ^ ((uint64_t)db * 0xD6E8FEB86659FD93ull));
    uint64_t y = mix64(x ^ ((uint64_t)db << 21) ^ 0x5851F42D4C957F2Dull);
    h0 += x;
    h1 += y;
}

// NVTX range for the host-side phases (build, lists, steps, windows), so that
// profilers can attribute launches; header-only NVTX3, a no-op without a tool.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// ---------------------------------------------------------------- buffers

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// Context shared by all entry points (defined in nd_capi.cu).
struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int32_t* d_err = nullptr;  // kErrWords device words
    int32_t* h_err = nullptr;  // pinned mirror
    int64_t launches = 0;
    std::string last_error;
    // scratch buffers of the neighbour-search pipeline, grown on demand
    DevBuf xyz, codes, codes_alt, perm, perm_alt, pos4, idx, keys, store, hist, counts, offsets,
        partial, pairs_i, pairs_j, pairs_d, misc, hash, leafpairs, ranges, tasks, compat;
    struct MDEngine* sim_cache = nullptr;  // engine re-used by nd_simulate
    bool no_alloc = false;                 // buffers are fixed slices: never grow them
};

// Grow `b` to at least `bytes` (contents are not preserved).
nd_status ensure(Ctx* c, DevBuf& b, size_t bytes);
nd_status cuda_fail(Ctx* c, cudaError_t e, const char* what);
nd_status check_launch(Ctx* c, const char* what);
// Synchronise the stream, read and clear the device error word.
nd_status sync_and_check(Ctx* c, const char* what);

// ------------------------------------------------ neighbour-search pipeline

struct TreeBuffers {
    int32_t n = 0, nL = 0, apl = 0;
    const int32_t* codes = nullptr;  // sorted codes (n)
    const int32_t* perm = nullptr;   // sorted -> original, 0-based (n)
    const float4* pos4 = nullptr;    // sorted positions, w = bits of 1-based index (n)
    const int32_t* idx = nullptr;    // sorted 1-based original index (n)
    float4* keys = nullptr;          // 2 float4 per node, nd_gridkey layout (nkeys)
    const int2* ranges = nullptr;    // leaf range of internal node nL + q at q - 1 (or null)
    int64_t nkeys = 0;
};

// Morton codes of n float3 positions (device, AoS) into codes + iota values.
// frame (ND_ORDER_SPATIAL only, may be NULL): host min[3], max[3] of the
// Hilbert grid instead of the positions' bounding box.
nd_status morton_codes(Ctx* c, const float* xyz, int32_t n, int32_t order, int32_t* codes,
                       int32_t* iota, const float* frame = nullptr);
// Stable LSD radix sort of (codes, vals) on `bits` low bits; results in codes/vals.
nd_status radix_sort_pairs(Ctx* c, uint32_t* keys, int32_t* vals, int32_t n, int bits);
// Full tree pipeline: codes -> sort -> gather -> leaf boxes -> Apetrei build.
nd_status build_tree(Ctx* c, const float* xyz_dev, int32_t n, float r, int32_t apl,
                     int32_t order, int32_t boxes, int64_t nkeys, bool overwrite_root,
                     TreeBuffers* out);
// Tree of new positions in the order (1-based original indices idx1) and with
// the sorted codes of an earlier build: same topology, new boxes (device
// arrays); the leaf-box half-width is r/2 (leafTreeData).
nd_status build_tree_kept(Ctx* c, const float* xyz_dev, int32_t n, float r, int32_t apl,
                          const int32_t* idx1, const int32_t* codes_sorted, int64_t nkeys,
                          TreeBuffers* out);
void root_overwrite(Ctx* c, float4* keys, int32_t nL);
// Exclusive int64 scan on the context stream; total written to *total_dev.
nd_status scan_exclusive(Ctx* c, const int64_t* in, int64_t* out, int64_t n, int64_t* total_dev);

// Pair emission over a built tree (kind: 0 = leaf path, 1 = per-atom path) is
// declared with the MD engine below.  pairs_common runs the whole pair-list
// pipeline on the context's buffers (host or device positions and outputs).
nd_status pairs_common(Ctx* c, const nd_bvh_spec* s, int32_t order, int32_t mode, int kind,
                       const float* xyz, bool host, int32_t* pi, int32_t* pj, float* pd,
                       int64_t capacity, int64_t* count, int32_t criterion = ND_CRIT_SQUARED);
nd_status pair_hash(Ctx* c, const int32_t* pi, const int32_t* pj, const float* pd, int64_t np,
                    uint64_t out[2]);

// Apetrei bottom-up build over already prepared leaf keys (used by the MD engine).
nd_status build_internal_nodes(Ctx* c, float4* keys, int32_t* store, const int32_t* codes_sorted,
                               int32_t nL, int32_t apl, int2* ranges = nullptr);

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace nd

// ------------------------------------------------------------- MD engine
namespace nd {
struct MDEngine;
nd_status md_create(Ctx* parent, const nd_md_params* p, int32_t n, const double* x,
                    const double* v, const double* q, const double* mass, bool host,
                    bool capture, MDEngine** out);
nd_status md_destroy(MDEngine* m);
nd_status md_create_batch(Ctx* parent, const nd_md_params* p, int32_t nsys, const nd_system* sys,
                          const double* x, const double* v, const double* q, const double* mass,
                          bool host, MDEngine** out);
nd_status md_energies(MDEngine* m, double* pot, double* kin);
nd_status md_step_times(MDEngine* m, int32_t steps, float* ms);
nd_status md_autotune(Ctx* parent, const nd_md_params* p, int32_t n, int32_t nsys,
                      const nd_system* sys, const double* x, const double* v, const double* q,
                      const double* mass, int32_t trial_steps, nd_md_params* best, double* sps);
nd_status md_reset(MDEngine* m, const double* x, const double* v, const double* q,
                   const double* mass, bool host);
bool md_compatible(MDEngine* m, const nd_md_params* p, int32_t n, bool has_q, bool has_m);
nd_status md_run(MDEngine* m, int64_t steps);
nd_status md_sync(MDEngine* m);
nd_status md_get(MDEngine* m, double* x, double* v, float* f, bool host);
nd_status md_energy(MDEngine* m, double* pot, double* kin);
nd_status md_stats(MDEngine* m, int64_t* steps, int64_t* rebuilds, int64_t* list_pairs,
                   int32_t* capacity);
int64_t md_launches_per_run(MDEngine* m, int64_t steps);
nd_status md_diagnostics(MDEngine* m, nd_md_diag* out);
nd_status md_list_pairs(MDEngine* m, int32_t* pi, int32_t* pj, uint8_t* near, int64_t cap,
                        int64_t* count);
nd_status md_set_thermostat(MDEngine* m, double temperature, double gamma, int32_t every);
nd_status md_set_log(MDEngine* m, int32_t every, int32_t frames);
nd_status md_log_count(MDEngine* m, int64_t* count);
nd_status md_log_read(MDEngine* m, int64_t first, int64_t nframes, double* out);
const char* md_last_error(MDEngine* m);
nd_status forces_pairs(Ctx* c, const nd_md_params* p, int32_t n, const double* x,
                       const double* q, const int32_t* pi, const int32_t* pj, int64_t np,
                       float* f, double* energy);
// Two-phase ordered emission: count (computes per-query offsets, syncs) then write.
// Squared-distance threshold of a pair criterion (ND_CRIT_*).
float pair_threshold(float r, int32_t criterion);
// Bug-compatible force_lennardjones! (kind 0) / force_coulomb! (kind 1) over a
// host pair list in list order; force: host N x 3 Float32.
nd_status compat_forces(Ctx* c, int kind, int32_t n, const int32_t* pi, const int32_t* pj,
                        const float* pd, int64_t np, const float* q, float* force);
// collect_objects(::GenericRandomCollector) on the device (host arrays out).
nd_status collect_objects(Ctx* c, const nd_collector* cl, uint64_t seed, float* x, float* v,
                          float* m, float* q, int64_t* pruned);
// simulate! as written over the all-pairs list (host arrays in and out).
nd_status compat_simulate(Ctx* c, const nd_compat_sim* spec, int32_t n, float* x, float* v,
                          float* force, const float* mass, const float* q, float* poslog);
nd_status count_pairs(Ctx* c, const TreeBuffers& t, float r2, int kind, int64_t* total);
nd_status write_pairs(Ctx* c, const TreeBuffers& t, float r2, int kind, int32_t* pi, int32_t* pj,
                      float* pd);
nd_status emit_unordered(Ctx* c, const TreeBuffers& t, float r, float r2, int32_t* pi,
                         int32_t* pj, float* pd, int64_t capacity, int64_t* total);

// ------------------------------------------------------------- adjoint
struct AdjEngine;
nd_status adj_create(Ctx* parent, const nd_md_params* p, int32_t n, const double* x0,
                     const double* v0, const double* q, const double* mass, const nd_adj_spec* s,
                     AdjEngine** out);
nd_status adj_destroy(AdjEngine* A);
nd_status adj_set_params(AdjEngine* A, double sigma, double epsilon);
nd_status adj_set_target(AdjEngine* A, const double* target);
nd_status adj_forward(AdjEngine* A, double* hist, double* loss);
nd_status adj_backward(AdjEngine* A, double* dx0, double* dv0, double* dsigma, double* deps);
nd_status adj_times(AdjEngine* A, float* fwd_ms, float* bwd_ms);
nd_status adj_final(AdjEngine* A, double* x);
const char* adj_last_error(AdjEngine* A);
}  // namespace nd
