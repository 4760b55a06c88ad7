// nd_bvh.cu -- LBVH neighbour search for sm_103a.
//
// Reference: src/Neighbors/BVHTraverse.jl (NaiveDynamics.jl).  The pipeline is
//   Morton codes (mortoncodes!, :237-288)  -> stable radix sort (sortperm, :570)
//   -> gather + leaf boxes (leafcluster_primitives :376-410 / cluster_primitives :341-375)
//   -> Apetrei bottom-up build with CAS (bvh_interior!, :704-846)
//   -> stackless rope traversal (leafneighbor_traverse :1236-1323,
//      neighbor_traverse :1125-1183) with pair emission.
// Everything that decides which pairs exist is computed with the reference's
// exact single-precision operation order (no FMA contraction, IEEE division and
// square root) so that codes, order, tree and pair list are bit-identical.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>

#include "nd_internal.cuh"

namespace nd {

// =================================================================== Morton

// mortoncodes! with K = Int32 (BVHTraverse.jl:259-284).
__global__ void k_morton_reference(const float* __restrict__ xyz, int32_t n, float binwidth,
                                   int32_t* __restrict__ codes, int32_t* __restrict__ iota,
                                   int32_t* err) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t magic[3] = {153391689, 306783378, 613566756};
    int32_t code = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float p = xyz[3 * (int64_t)i + d];
        if (!isfinite(p)) { set_error(err, ND_ERR_NONFINITE, i); code = 0; break; }
        float q = floorf(__fdiv_rn(p, binwidth));
        // trunc(Int32, ::Float32) accepts -2^31 <= q < 2^31 (Julia Base float.jl)
        if (!(q >= -2147483648.0f && q < 2147483648.0f)) { set_error(err, ND_ERR_RANGE, i); code = 0; break; }
        int32_t qi = (int32_t)q;
        int32_t yin = qi & magic[d];
        int32_t yang = qi | ~magic[d];
        code |= (yin & yang);
    }
    codes[i] = code;
    if (iota) iota[i] = i;
}

// Bounding box of the positions (order-preserving uint atomics), used by the
// spatial code.  bbox[0..2] = min keys, bbox[3..5] = max keys.
__global__ void k_bbox(const float* __restrict__ xyz, int32_t n, uint32_t* bbox, int32_t* err) {
    uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu};
    uint32_t mx[3] = {0u, 0u, 0u};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float p = xyz[3 * i + d];
            if (!isfinite(p)) { set_error(err, ND_ERR_NONFINITE, (int32_t)i); continue; }
            uint32_t o = f2o(p);
            mn[d] = min(mn[d], o);
            mx[d] = max(mx[d], o);
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int s = 16; s > 0; s >>= 1) {
            mn[d] = min(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], s));
            mx[d] = max(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], s));
        }
    }
    // block reduction first: one atomic per block and component
    __shared__ uint32_t s_b[32][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int d = 0; d < 3; ++d) { s_b[warp][d] = mn[d]; s_b[warp][3 + d] = mx[d]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        uint32_t v = s_b[0][k];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = k < 3 ? min(v, s_b[w][k]) : max(v, s_b[w][k]);
        if (k < 3) atomicMin(&bbox[k], v);
        else atomicMax(&bbox[k], v);
    }
}

__global__ void k_bbox_init(uint32_t* bbox) {
    if (threadIdx.x < 6) bbox[threadIdx.x] = threadIdx.x < 3 ? 0xffffffffu : 0u;
}

// A given frame in place of the bounding box.
__global__ void k_bbox_set(uint32_t* bbox, float x0, float y0, float z0, float x1, float y1,
                           float z1) {
    const float v[6] = {x0, y0, z0, x1, y1, z1};
    if (threadIdx.x < 6) bbox[threadIdx.x] = f2o(v[threadIdx.x]);
}

// Spatial code: 3-D Hilbert index over the bounding box, 1024 bins per axis.
__global__ void k_morton_spatial(const float* __restrict__ xyz, int32_t n,
                                 const uint32_t* __restrict__ bbox, int32_t* __restrict__ codes,
                                 int32_t* __restrict__ iota) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t q[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float lo = o2f(bbox[d]), hi = o2f(bbox[3 + d]);
        float ext = __fsub_rn(hi, lo);
        float s = ext > 0.0f ? __fdiv_rn(1024.0f, ext) : 0.0f;
        float t = floorf(__fmul_rn(__fsub_rn(xyz[3 * (int64_t)i + d], lo), s));
        int32_t qi = (t < 0.0f) ? 0 : (t > 1023.0f ? 1023 : (int32_t)t);
        q[d] = (uint32_t)qi;
    }
    codes[i] = (int32_t)hilbert3_10(q[0], q[1], q[2]);
    if (iota) iota[i] = i;
}

nd_status morton_codes(Ctx* c, const float* xyz, int32_t n, int32_t order, int32_t* codes,
                       int32_t* iota, const float* frame) {
    if (n <= 0) return ND_OK;
    const int T = 256;
    if (order == ND_ORDER_SPATIAL) {
        nd_status st = ensure(c, c->misc, 64);
        if (st) return st;
        if (frame) {
            k_bbox_set<<<1, 32, 0, c->stream>>>((uint32_t*)c->misc.p, frame[0], frame[1], frame[2],
                                                frame[3], frame[4], frame[5]);
            c->launches++;
        } else {
            k_bbox_init<<<1, 32, 0, c->stream>>>((uint32_t*)c->misc.p);
            c->launches++;
            int blocks = (int)std::min<int64_t>(cdiv(n, T), 152 * 8);
            k_bbox<<<blocks, T, 0, c->stream>>>(xyz, n, (uint32_t*)c->misc.p, c->d_err);
            c->launches++;
        }
        k_morton_spatial<<<(int)cdiv(n, T), T, 0, c->stream>>>(xyz, n, (const uint32_t*)c->misc.p,
                                                              codes, iota);
        c->launches++;
    } else {
        const float binwidth = (float)(1.0 / 1023.0);  // Float32(1/1023), BVHTraverse.jl:184
        k_morton_reference<<<(int)cdiv(n, T), T, 0, c->stream>>>(xyz, n, binwidth, codes, iota,
                                                                c->d_err);
        c->launches++;
    }
    return check_launch(c, "morton");
}

// ================================================================ radix sort
// Stable LSD radix sort, 8-bit digits, reduce-then-scan (no inter-CTA waiting):
//   upsweep: per-tile digit histograms, digit-major;
//   scan:    per-digit exclusive scan over tiles + digit totals;
//   scatter: stable in-tile ranks (warp match + per-warp prefix) -> global slot.

constexpr int RS_BINS = 256;
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
static_assert(RS_THREADS == RS_BINS, "scatter maps one thread per digit");

__global__ void __launch_bounds__(RS_THREADS)
    k_rs_upsweep(const uint32_t* __restrict__ keys, int32_t n, int shift,
                 uint32_t* __restrict__ hist, int32_t ntiles) {
    __shared__ uint32_t sh[RS_BINS];
    sh[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * RS_TILE;
    const unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < RS_ITEMS; ++k) {
        int64_t idx = base + k * RS_THREADS + threadIdx.x;
        bool valid = idx < n;
        uint32_t dg = valid ? ((keys[idx] >> shift) & 0xffu) : 0x100u;
        unsigned peers = __match_any_sync(0xffffffffu, dg);
        if (valid && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(&sh[dg], (uint32_t)__popc(peers));
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = sh[threadIdx.x];
}

__device__ __forceinline__ uint32_t block_excl_scan_256(uint32_t v, uint32_t* s_warp,
                                                        uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, s);
        if (lane >= s) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0u;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, s);
            if (lane >= s) w += y;
        }
        if (lane < (int)(blockDim.x >> 5)) s_warp[lane] = w;  // inclusive warp prefix
    }
    __syncthreads();
    uint32_t wp = warp ? s_warp[warp - 1] : 0u;
    if (total) *total = s_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return wp + x - v;
}

// One CTA per digit: exclusive scan of that digit's per-tile counts.
__global__ void __launch_bounds__(RS_THREADS)
    k_rs_scan(uint32_t* __restrict__ hist, int32_t ntiles, uint32_t* __restrict__ totals) {
    __shared__ uint32_t s_warp[32];
    uint32_t* h = hist + (int64_t)blockIdx.x * ntiles;
    uint32_t carry = 0;
    for (int32_t b = 0; b < ntiles; b += RS_THREADS) {
        int32_t i = b + threadIdx.x;
        uint32_t v = i < ntiles ? h[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_excl_scan_256(v, s_warp, &tot);
        if (i < ntiles) h[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(RS_THREADS)
    k_rs_scatter(const uint32_t* __restrict__ kin, const int32_t* __restrict__ vin,
                 uint32_t* __restrict__ kout, int32_t* __restrict__ vout, int32_t n, int shift,
                 const uint32_t* __restrict__ hist, const uint32_t* __restrict__ totals,
                 int32_t ntiles) {
    constexpr int W = RS_THREADS / 32;
    __shared__ uint32_t s_base[RS_BINS];
    __shared__ uint32_t s_run[RS_BINS];
    __shared__ uint32_t s_wh[W][RS_BINS];
    __shared__ uint32_t s_warp[32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t ex = block_excl_scan_256(totals[t], s_warp, nullptr);
    s_base[t] = ex + hist[(int64_t)t * ntiles + blockIdx.x];
    s_run[t] = 0;
    const unsigned lt = (1u << lane) - 1u;
    int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int k = 0; k < RS_ITEMS; ++k) {
#pragma unroll
        for (int w = 0; w < W; ++w) s_wh[w][t] = 0;
        __syncthreads();
        int64_t idx = base + k * RS_THREADS + t;
        bool valid = idx < n;
        uint32_t key = valid ? kin[idx] : 0u;
        int32_t val = valid ? vin[idx] : 0;
        uint32_t dg = valid ? ((key >> shift) & 0xffu) : 0x100u;
        unsigned peers = __match_any_sync(0xffffffffu, dg);
        int rank = __popc(peers & lt);
        if (valid && lane == __ffs(peers) - 1) s_wh[warp][dg] = (uint32_t)__popc(peers);
        __syncthreads();
        {
            uint32_t run = s_run[t];
#pragma unroll
            for (int w = 0; w < W; ++w) {
                uint32_t cnt = s_wh[w][t];
                s_wh[w][t] = run;
                run += cnt;
            }
            s_run[t] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = s_base[dg] + s_wh[warp][dg] + (uint32_t)rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
    }
}

nd_status radix_sort_pairs(Ctx* c, uint32_t* keys, int32_t* vals, int32_t n, int bits) {
    if (n <= 1) return ND_OK;
    int32_t ntiles = (int32_t)cdiv(n, RS_TILE);
    nd_status st;
    if ((st = ensure(c, c->codes_alt, sizeof(uint32_t) * (size_t)n))) return st;
    if ((st = ensure(c, c->perm_alt, sizeof(int32_t) * (size_t)n))) return st;
    if ((st = ensure(c, c->hist, sizeof(uint32_t) * ((size_t)RS_BINS * ntiles + RS_BINS))))
        return st;
    uint32_t* hist = (uint32_t*)c->hist.p;
    uint32_t* totals = hist + (size_t)RS_BINS * ntiles;
    uint32_t* ka = keys;
    int32_t* va = vals;
    uint32_t* kb = (uint32_t*)c->codes_alt.p;
    int32_t* vb = (int32_t*)c->perm_alt.p;
    int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        k_rs_upsweep<<<ntiles, RS_THREADS, 0, c->stream>>>(ka, n, shift, hist, ntiles);
        k_rs_scan<<<RS_BINS, RS_THREADS, 0, c->stream>>>(hist, ntiles, totals);
        k_rs_scatter<<<ntiles, RS_THREADS, 0, c->stream>>>(ka, va, kb, vb, n, shift, hist, totals,
                                                          ntiles);
        c->launches += 3;
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys) {
        cudaMemcpyAsync(keys, ka, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, c->stream);
        cudaMemcpyAsync(vals, va, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, c->stream);
    }
    return check_launch(c, "radix sort");
}

// ============================================================== leaf boxes

// Gather sorted positions and build leaf boxes: leafcluster_primitives
// (BVHTraverse.jl:376-410, h = r/2) or cluster_primitives (:341-375, h = r).
// pos4.w carries the 1-based original index (bit pattern).
__global__ void k_leaf_boxes(const float* __restrict__ xyz, const int32_t* __restrict__ perm,
                             int32_t nL, int32_t apl, float h, float4* __restrict__ pos4,
                             int32_t* __restrict__ idx, float4* __restrict__ keys) {
    int32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= nL) return;
    int64_t bird = (int64_t)leaf * apl;
    float mn[3], mx[3];
    for (int32_t a = 0; a < apl; ++a) {
        int32_t o = perm[bird + a];
        float p[3] = {xyz[3 * (int64_t)o], xyz[3 * (int64_t)o + 1], xyz[3 * (int64_t)o + 2]};
        pos4[bird + a] = make_float4(p[0], p[1], p[2], __int_as_float(o + 1));
        idx[bird + a] = o + 1;
        if (a == 0) {
#pragma unroll
            for (int d = 0; d < 3; ++d) { mn[d] = __fsub_rn(p[d], h); mx[d] = __fadd_rn(p[d], h); }
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            mn[d] = jl_min(mn[d], __fsub_rn(p[d], h));
            mx[d] = jl_max(mx[d], __fadd_rn(p[d], h));
        }
    }
    keys[2 * (int64_t)leaf] = make_float4(mn[0], mn[1], mn[2], mx[0]);
    keys[2 * (int64_t)leaf + 1] = make_float4(mx[1], mx[2], __int_as_float(0), __int_as_float(0));
}

// ==================================================================== build

// exptdelta (BVHTraverse.jl:677-696), 1-based leaf index, Int32 wrap-around.
__device__ __forceinline__ int32_t delta_ref(int32_t i, const int32_t* __restrict__ code,
                                             int32_t nL, int32_t apl) {
    if (i >= nL || i < 1) return INT32_MAX;
    int32_t a = __ldg(&code[(int64_t)(i - 1) * apl]);
    int32_t b = __ldg(&code[(int64_t)i * apl]);
    uint32_t x = (uint32_t)(a ^ b);
    uint32_t add = (x == 0u) ? (0x80000000u + (uint32_t)(i ^ (i + 1))) : 0u;
    return (int32_t)(x + add - 1u);
}

__device__ __forceinline__ void load_box_cg(const float4* keys, int32_t node /*1-based*/,
                                            float mn[3], float mx[3]) {
    float4 a = __ldcg(&keys[2 * (int64_t)(node - 1)]);
    float4 b = __ldcg(&keys[2 * (int64_t)(node - 1) + 1]);
    mn[0] = a.x; mn[1] = a.y; mn[2] = a.z;
    mx[0] = a.w; mx[1] = b.x; mx[2] = b.y;
}

// bvh_interior! (BVHTraverse.jl:704-846), one thread per leaf.  The second
// thread to reach an internal node (the CAS on store[split] returns non-zero)
// merges the sibling box and continues upward.  __threadfence() before the CAS
// publishes this thread's node writes; the fence after a successful read of a
// non-zero slot orders the sibling-box loads, which bypass L1 (ld.cg).  No
// thread ever waits on another, so the kernel cannot hang; a climb longer than
// nL levels flags ND_ERR_INTERNAL.  ranges (may be null): leaf range
// [first, last] of internal node nL + q at ranges[q - 1].
__global__ void k_bvh_build(float4* keys, int32_t* store, const int32_t* __restrict__ code,
                            int32_t nL, int32_t apl, int2* ranges, int32_t* err) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > nL) return;
    int32_t rangel = i, ranger = i;
    int32_t dell = delta_ref(rangel - 1, code, nL, apl);
    int32_t delr = delta_ref(ranger, code, nL, apl);
    float bmin[3], bmax[3];
    load_box_cg(keys, i, bmin, bmax);
    int32_t lskip;
    if (i == nL) {
        lskip = 0;
    } else {
        int32_t ir = i + 1;
        lskip = (delr < delta_ref(ir, code, nL, apl)) ? ir : nL + ir;
    }
    reinterpret_cast<int32_t*>(&keys[2 * (int64_t)(i - 1) + 1])[3] = lskip;

    for (int32_t guard = 0; guard <= nL + 1; ++guard) {
        int32_t leftChild;
        int32_t sib;
        if (delr < dell) {
            leftChild = i;
            int32_t split = ranger;
            __threadfence();
            ranger = atomicCAS(&store[split - 1], 0, rangel);
            if (ranger == 0) return;
            __threadfence();
            delr = delta_ref(ranger, code, nL, apl);
            sib = split + 1;
            if (sib != ranger) sib = nL + sib;
        } else {
            int32_t split = rangel - 1;
            __threadfence();
            rangel = atomicCAS(&store[split - 1], 0, ranger);
            if (rangel == 0) return;
            __threadfence();
            dell = delta_ref(rangel - 1, code, nL, apl);
            leftChild = split;
            if (leftChild != rangel) leftChild = nL + leftChild;
            sib = leftChild;
        }
        float smin[3], smax[3];
        load_box_cg(keys, sib, smin, smax);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            bmax[d] = jl_max(smax[d], bmax[d]);
            bmin[d] = jl_min(smin[d], bmin[d]);
        }
        int32_t q = (delr < dell) ? ranger : rangel;
        int32_t parent = nL + q;
        if (ranges) ranges[q - 1] = make_int2(rangel, ranger);
        int32_t skip;
        if (ranger == nL) {
            skip = 0;
        } else {
            int32_t r = ranger + 1;
            skip = (delr < delta_ref(r, code, nL, apl)) ? r : nL + r;
        }
        __stcg(&keys[2 * (int64_t)(parent - 1)], make_float4(bmin[0], bmin[1], bmin[2], bmax[0]));
        __stcg(&keys[2 * (int64_t)(parent - 1) + 1],
               make_float4(bmax[1], bmax[2], __int_as_float(leftChild), __int_as_float(skip)));
        i = parent;
        if (i == nL + 1) return;
    }
    set_error(err, ND_ERR_INTERNAL, i);
}

__global__ void k_root_overwrite(float4* keys, int32_t nL) {
    // bounding_volume_hierarchy! (BVHTraverse.jl:856-858) forces the root box to [0,1]^3.
    float4 b = keys[2 * (int64_t)nL + 1];
    keys[2 * (int64_t)nL] = make_float4(0.f, 0.f, 0.f, 1.f);
    keys[2 * (int64_t)nL + 1] = make_float4(1.f, 1.f, b.z, b.w);
}

nd_status build_internal_nodes(Ctx* c, float4* keys, int32_t* store, const int32_t* codes,
                               int32_t nL, int32_t apl, int2* ranges) {
    cudaError_t e = cudaMemsetAsync(store, 0, sizeof(int32_t) * (size_t)(nL - 1), c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "store reset");
    k_bvh_build<<<(int)cdiv(nL, 256), 256, 0, c->stream>>>(keys, store, codes, nL, apl, ranges,
                                                            c->d_err);
    c->launches++;
    return check_launch(c, "bvh build");
}

nd_status build_tree(Ctx* c, const float* xyz_dev, int32_t n, float r, int32_t apl,
                     int32_t order, int32_t boxes, int64_t nkeys, bool overwrite_root,
                     TreeBuffers* out) {
    int32_t nL = n / apl;
    nd_status st;
    if ((st = ensure(c, c->codes, sizeof(int32_t) * (size_t)n))) return st;
    if ((st = ensure(c, c->perm, sizeof(int32_t) * (size_t)n))) return st;
    if ((st = ensure(c, c->pos4, sizeof(float4) * (size_t)n))) return st;
    if ((st = ensure(c, c->idx, sizeof(int32_t) * (size_t)n))) return st;
    if ((st = ensure(c, c->keys, 32 * (size_t)nkeys))) return st;
    if ((st = ensure(c, c->store, sizeof(int32_t) * (size_t)std::max(nL - 1, 1)))) return st;
    int32_t* codes = (int32_t*)c->codes.p;
    int32_t* perm = (int32_t*)c->perm.p;
    if ((st = morton_codes(c, xyz_dev, n, order, codes, perm))) return st;
    if ((st = radix_sort_pairs(c, (uint32_t*)codes, perm, n, 30))) return st;
    float4* keys = (float4*)c->keys.p;
    cudaError_t e = cudaMemsetAsync(keys, 0, 32 * (size_t)nkeys, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "keys reset");
    float h = (boxes == ND_BOX_LEAF) ? r / 2.0f : r;
    k_leaf_boxes<<<(int)cdiv(nL, 128), 128, 0, c->stream>>>(xyz_dev, perm, nL, apl, h,
                                                           (float4*)c->pos4.p,
                                                           (int32_t*)c->idx.p, keys);
    c->launches++;
    if ((st = check_launch(c, "leaf boxes"))) return st;
    // leaf ranges of the internal nodes, for the split walks of the two-phase
    // emission (not kept by the allocation-free entry point)
    int2* ranges = nullptr;
    if (!c->no_alloc) {
        if ((st = ensure(c, c->ranges, sizeof(int2) * (size_t)std::max(nL - 1, 1)))) return st;
        ranges = (int2*)c->ranges.p;
    }
    if ((st = build_internal_nodes(c, keys, (int32_t*)c->store.p, codes, nL, apl, ranges)))
        return st;
    if (overwrite_root) {
        k_root_overwrite<<<1, 1, 0, c->stream>>>(keys, nL);
        c->launches++;
    }
    out->n = n;
    out->nL = nL;
    out->apl = apl;
    out->codes = codes;
    out->perm = perm;
    out->pos4 = (const float4*)c->pos4.p;
    out->idx = (const int32_t*)c->idx.p;
    out->keys = keys;
    out->ranges = ranges;
    out->nkeys = nkeys;
    return check_launch(c, "tree");
}

// Sorted -> original permutation (0-based) from the 1-based original indices
// of a kept order.
__global__ void k_kept_perm(const int32_t* __restrict__ idx1, int32_t n, int32_t* __restrict__ perm) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) perm[i] = idx1[i] - 1;
}

// Tree of new positions in a kept order: the sorted codes and the order of an
// earlier build are reused, so the Apetrei build (which depends on the sorted
// codes only) reproduces that build's topology, and the leaf and internal
// boxes are those of the new positions -- the refit that TreeData!
// (src/Neighbors/BVHTraverse.jl:601-655) intends between rebuilds.  idx1 and
// codes are device arrays (1-based original index and code, sorted order).
nd_status build_tree_kept(Ctx* c, const float* xyz_dev, int32_t n, float r, int32_t apl,
                          const int32_t* idx1, const int32_t* codes_sorted, int64_t nkeys,
                          TreeBuffers* out) {
    int32_t nL = n / apl;
    nd_status st;
    if ((st = ensure(c, c->perm, sizeof(int32_t) * (size_t)n))) return st;
    if ((st = ensure(c, c->pos4, sizeof(float4) * (size_t)n))) return st;
    if ((st = ensure(c, c->idx, sizeof(int32_t) * (size_t)n))) return st;
    if ((st = ensure(c, c->keys, 32 * (size_t)nkeys))) return st;
    if ((st = ensure(c, c->store, sizeof(int32_t) * (size_t)std::max(nL - 1, 1)))) return st;
    if ((st = ensure(c, c->ranges, sizeof(int2) * (size_t)std::max(nL - 1, 1)))) return st;
    int32_t* perm = (int32_t*)c->perm.p;
    k_kept_perm<<<(unsigned)cdiv(n, 256), 256, 0, c->stream>>>(idx1, n, perm);
    c->launches++;
    float4* keys = (float4*)c->keys.p;
    cudaError_t e = cudaMemsetAsync(keys, 0, 32 * (size_t)nkeys, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "keys reset");
    k_leaf_boxes<<<(int)cdiv(nL, 128), 128, 0, c->stream>>>(xyz_dev, perm, nL, apl, r / 2.0f,
                                                           (float4*)c->pos4.p,
                                                           (int32_t*)c->idx.p, keys);
    c->launches++;
    if ((st = check_launch(c, "kept leaf boxes"))) return st;
    int2* ranges = (int2*)c->ranges.p;
    if ((st = build_internal_nodes(c, keys, (int32_t*)c->store.p, codes_sorted, nL, apl, ranges)))
        return st;
    out->n = n;
    out->nL = nL;
    out->apl = apl;
    out->codes = codes_sorted;
    out->perm = perm;
    out->pos4 = (const float4*)c->pos4.p;
    out->idx = (const int32_t*)c->idx.p;
    out->keys = keys;
    out->ranges = ranges;
    out->nkeys = nkeys;
    return check_launch(c, "kept tree");
}

// bounding_volume_hierarchy!'s root-box overwrite on a built tree.
void root_overwrite(Ctx* c, float4* keys, int32_t nL) {
    k_root_overwrite<<<1, 1, 0, c->stream>>>(keys, nL);
    c->launches++;
}

// ==================================================================== scan

constexpr int SC_THREADS = 1024;
constexpr int SC_ITEMS = 4;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

__global__ void __launch_bounds__(SC_THREADS)
    k_scan_tile(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                int64_t* __restrict__ partial) {
    __shared__ int64_t s_warp[32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int64_t base = (int64_t)blockIdx.x * SC_TILE + (int64_t)t * SC_ITEMS;
    int64_t v[SC_ITEMS];
    int64_t sum = 0;
#pragma unroll
    for (int k = 0; k < SC_ITEMS; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        sum += v[k];
    }
    int64_t x = sum;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, s);
        if (lane >= s) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t w = s_warp[lane];
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, w, s);
            if (lane >= s) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    int64_t run = (warp ? s_warp[warp - 1] : 0) + x - sum;
#pragma unroll
    for (int k = 0; k < SC_ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (t == SC_THREADS - 1 && partial) partial[blockIdx.x] = s_warp[31];
}

__global__ void k_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ add) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += add[i / SC_TILE];
}

__global__ void k_scan_total(const int64_t* in, const int64_t* out, int64_t n, int64_t* total) {
    *total = n > 0 ? in[n - 1] + out[n - 1] : 0;
}

static nd_status scan_rec(Ctx* c, const int64_t* in, int64_t* out, int64_t n, int64_t* scratch,
                          size_t scratch_elems) {
    int64_t nb = cdiv(n, SC_TILE);
    if (nb <= 1) {
        k_scan_tile<<<1, SC_THREADS, 0, c->stream>>>(in, out, n, nullptr);
        c->launches++;
        return check_launch(c, "scan");
    }
    if ((size_t)(2 * nb) > scratch_elems) return ND_ERR_INTERNAL;
    int64_t* part = scratch;
    int64_t* part_scan = scratch + nb;
    k_scan_tile<<<(unsigned)nb, SC_THREADS, 0, c->stream>>>(in, out, n, part);
    c->launches++;
    nd_status st = scan_rec(c, part, part_scan, nb, scratch + 2 * nb, scratch_elems - 2 * nb);
    if (st) return st;
    k_scan_add<<<(unsigned)cdiv(n, 256), 256, 0, c->stream>>>(out, n, part_scan);
    c->launches++;
    return check_launch(c, "scan add");
}

nd_status scan_exclusive(Ctx* c, const int64_t* in, int64_t* out, int64_t n, int64_t* total_dev) {
    if (n <= 0) {
        cudaMemsetAsync(total_dev, 0, sizeof(int64_t), c->stream);
        return ND_OK;
    }
    size_t need = 4 * (size_t)cdiv(n, SC_TILE) + 64;
    nd_status st = ensure(c, c->partial, sizeof(int64_t) * need);
    if (st) return st;
    st = scan_rec(c, in, out, n, (int64_t*)c->partial.p, need);
    if (st) return st;
    k_scan_total<<<1, 1, 0, c->stream>>>(in, out, n, total_dev);
    c->launches++;
    return check_launch(c, "scan total");
}

// =============================================================== traversal

struct Node {
    float mnx, mny, mnz, mxx, mxy, mxz;
    int32_t left, skip;
};

__device__ __forceinline__ Node load_node(const float4* __restrict__ keys, int32_t k /*1-based*/) {
    float4 a = __ldg(&keys[2 * (int64_t)(k - 1)]);
    float4 b = __ldg(&keys[2 * (int64_t)(k - 1) + 1]);
    Node nd_;
    nd_.mnx = a.x; nd_.mny = a.y; nd_.mnz = a.z; nd_.mxx = a.w; nd_.mxy = b.x; nd_.mxz = b.y;
    nd_.left = __float_as_int(b.z);
    nd_.skip = __float_as_int(b.w);
    return nd_;
}

// aabb_overlap_test (BVHTraverse.jl:1094-1098), strict on all three axes.
__device__ __forceinline__ bool overlap(const Node& a, const Node& b) {
    return (a.mnx < b.mxx) & (a.mxx > b.mnx) & (a.mny < b.mxy) & (a.mxy > b.mny) &
           (a.mnz < b.mxz) & (a.mxz > b.mnz);
}

// Rounding slack of leaf a's box coordinates: 8 ulps of the largest.
__device__ __forceinline__ float leaf_slack(const Node& a) {
    const float mag = fmaxf(fmaxf(fmaxf(fabsf(a.mnx), fabsf(a.mxx)), fmaxf(fabsf(a.mny), fabsf(a.mxy))),
                            fmaxf(fabsf(a.mnz), fabsf(a.mxz)));
    return mag * 9.5367431640625e-7f;  // 8 * 2^-23
}

// Whether two leaves whose key boxes (atom boxes -/+ r/2) overlap can hold a
// pair within r: the per-axis gaps of the atom boxes (key-box gap + r, each
// lowered by the rounding slack of the -/+ r/2) must have a Euclidean norm
// below r (r2g = r^2 widened a little: a filter, the distance test decides).
// Boxes that overlap on every axis only bound each gap by r; this drops the
// leaf pairs diagonally apart.
__device__ __forceinline__ bool leaf_gap_ok(const Node& a, const Node& b, float r, float r2g,
                                            float slack) {
    const float gx = fmaxf(fmaxf(a.mnx - b.mxx, b.mnx - a.mxx) + r - slack, 0.0f);
    const float gy = fmaxf(fmaxf(a.mny - b.mxy, b.mny - a.mxy) + r - slack, 0.0f);
    const float gz = fmaxf(fmaxf(a.mnz - b.mxz, b.mnz - a.mxz) + r - slack, 0.0f);
    return gx * gx + gy * gy + gz * gz < r2g;
}

// Emission sinks.  COUNT counts; WRITE writes at a running cursor; ATOMIC
// reserves chunks of a global cursor (warp-aggregated) as pairs appear.
struct SinkCount {
    int64_t n = 0;
    __device__ __forceinline__ void push(int32_t, int32_t, float) { ++n; }
};
struct SinkWrite {
    int32_t* pi; int32_t* pj; float* pd;
    int64_t cur;
    __device__ __forceinline__ void push(int32_t i, int32_t j, float d) {
        pi[cur] = i; pj[cur] = j; pd[cur] = d; ++cur;
    }
};

// Test query atoms qa[0..na) against target atoms tb[0..nb): every (a, b) with
// d^2 < r^2 in the reference's order (a outer, b inner), or, when `tri`, the
// intra-leaf pairs a < b (onecluster_proximitytest!, BVHTraverse.jl:1021-1040).
template <class Sink>
__device__ __forceinline__ void leaf_pairs_generic(const float4* __restrict__ pos, int64_t A,
                                                   int64_t B, int32_t apl, float r2, bool tri,
                                                   Sink& s) {
    for (int32_t i = 0; i < apl; ++i) {
        float4 a = __ldg(&pos[A + i]);
        for (int32_t j = tri ? i + 1 : 0; j < apl; ++j) {
            float4 b = __ldg(&pos[B + j]);
            float d2 = dist2_ref(a.x, a.y, a.z, b.x, b.y, b.z);
            if (d2 < r2) s.push(__float_as_int(a.w), __float_as_int(b.w), __fsqrt_rn(d2));
        }
    }
}

template <int APL, class Sink>
__device__ __forceinline__ void leaf_pairs_fixed(const float4 (&qa)[APL],
                                                 const float4* __restrict__ pos, int64_t B,
                                                 float r2, Sink& s) {
    float4 tb[APL];
#pragma unroll
    for (int j = 0; j < APL; ++j) tb[j] = __ldg(&pos[B + j]);
#pragma unroll
    for (int i = 0; i < APL; ++i)
#pragma unroll
        for (int j = 0; j < APL; ++j) {
            float d2 = dist2_ref(qa[i].x, qa[i].y, qa[i].z, tb[j].x, tb[j].y, tb[j].z);
            if (d2 < r2) s.push(__float_as_int(qa[i].w), __float_as_int(tb[j].w), __fsqrt_rn(d2));
        }
}

// leafneighbor_traverse (BVHTraverse.jl:1236-1323) for one query leaf q (1-based).
// A rope walk visits every node at most once; a longer walk or a node index
// outside [1, 2nL-1] can only come from a corrupted tree and is reported
// instead of looping.
#define ND_WALK_GUARD(t, nnodes, visits, err, who)                          \
    if ((t) < 1 || (t) > (nnodes) || ++(visits) > (nnodes)) {               \
        set_error((err), ND_ERR_INTERNAL, (who));                           \
        break;                                                              \
    }

template <int APL, class Sink>
__device__ __forceinline__ void leaf_query(int32_t q, const float4* __restrict__ keys,
                                           const float4* __restrict__ pos, int32_t apl, float r2,
                                           int32_t nnodes, int32_t* err, Sink& s) {
    Node ql = load_node(keys, q);
    int32_t visits = 0;
    int64_t A = (int64_t)(q - 1) * apl;
    if constexpr (APL > 0) {
        float4 qa[APL];
#pragma unroll
        for (int i = 0; i < APL; ++i) qa[i] = __ldg(&pos[A + i]);
#pragma unroll
        for (int i = 0; i < APL - 1; ++i)
#pragma unroll
            for (int j = i + 1; j < APL; ++j) {
                float d2 = dist2_ref(qa[i].x, qa[i].y, qa[i].z, qa[j].x, qa[j].y, qa[j].z);
                if (d2 < r2) s.push(__float_as_int(qa[i].w), __float_as_int(qa[j].w), __fsqrt_rn(d2));
            }
        int32_t t = ql.skip;
        while (t != 0) {
            ND_WALK_GUARD(t, nnodes, visits, err, q)
            Node nd_ = load_node(keys, t);
            if (overlap(ql, nd_)) {
                if (nd_.left == 0) {
                    leaf_pairs_fixed<APL>(qa, pos, (int64_t)(t - 1) * APL, r2, s);
                    t = nd_.skip;
                } else {
                    t = nd_.left;
                }
            } else {
                t = nd_.skip;
            }
        }
    } else {
        leaf_pairs_generic(pos, A, A, apl, r2, true, s);
        int32_t t = ql.skip;
        while (t != 0) {
            ND_WALK_GUARD(t, nnodes, visits, err, q)
            Node nd_ = load_node(keys, t);
            if (overlap(ql, nd_)) {
                if (nd_.left == 0) {
                    leaf_pairs_generic(pos, A, (int64_t)(t - 1) * apl, apl, r2, false, s);
                    t = nd_.skip;
                } else {
                    t = nd_.left;
                }
            } else {
                t = nd_.skip;
            }
        }
    }
}

// neighbor_traverse (BVHTraverse.jl:1143-1181) for one query atom qi (1-based, sorted).
template <class Sink>
__device__ __forceinline__ void atom_query(int32_t qi, const float4* __restrict__ keys,
                                           const float4* __restrict__ pos, int32_t apl, float r2,
                                           int32_t nnodes, int32_t* err, Sink& s) {
    float4 p = __ldg(&pos[qi - 1]);
    int32_t t = (qi + apl - 1) / apl;
    int32_t visits = 0;
    while (t != 0) {
        ND_WALK_GUARD(t, nnodes, visits, err, qi)
        Node nd_ = load_node(keys, t);
        bool in = (nd_.mnx < p.x) & (p.x < nd_.mxx) & (nd_.mny < p.y) & (p.y < nd_.mxy) &
                  (nd_.mnz < p.z) & (p.z < nd_.mxz);
        if (in) {
            if (nd_.left == 0) {
                int32_t low = (t - 1) * apl + 1;
                for (int32_t e = 1; e <= apl; ++e) {
                    int32_t sidx = low + e - 1;
                    if (qi < e + low) {
                        float4 b = __ldg(&pos[sidx - 1]);
                        if (__float_as_int(p.w) != __float_as_int(b.w)) {
                            float d2 = dist2_ref(p.x, p.y, p.z, b.x, b.y, b.z);
                            if (d2 < r2) s.push(__float_as_int(p.w), __float_as_int(b.w), __fsqrt_rn(d2));
                        }
                    }
                }
                t = nd_.skip;
            } else {
                t = nd_.left;
            }
        } else {
            t = nd_.skip;
        }
    }
}

template <int APL>
__global__ void __launch_bounds__(128)
    k_leaf_count(const float4* __restrict__ keys, const float4* __restrict__ pos, int32_t nL,
                 int32_t apl, float r2, int64_t* __restrict__ counts, int32_t* err) {
    int32_t q = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (q > nL) return;
    SinkCount s;
    leaf_query<APL>(q, keys, pos, apl, r2, 2 * nL - 1, err, s);
    counts[q - 1] = s.n;
}

template <int APL>
__global__ void __launch_bounds__(128)
    k_leaf_write(const float4* __restrict__ keys, const float4* __restrict__ pos, int32_t nL,
                 int32_t apl, float r2, const int64_t* __restrict__ offsets, int32_t* pi,
                 int32_t* pj, float* pd, int32_t* err) {
    int32_t q = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (q > nL) return;
    SinkWrite s{pi, pj, pd, offsets[q - 1]};
    leaf_query<APL>(q, keys, pos, apl, r2, 2 * nL - 1, err, s);
}

// One-pass emission, warp-cooperative (atomsperleaf 4; the pair multiset of
// leafneighbor_traverse in an order decided at run time).  A warp
// takes 32 consecutive query leaves and walks the tree ONCE, from the skip
// rope of its first leaf, pruning with the union of its lanes' boxes; at
// every leaf t it reaches, each lane runs leafneighbor_traverse's leaf test
// for its own leaf q (t > q, strict box overlap -- the leaves a rope walk
// from q's skip would accept, since a box overlapping t overlaps all of t's
// ancestors) and the 4 x 4 distance tests.  Lanes stay converged, node loads
// are broadcast, and the pairs are ballot-compacted into a shared-memory
// buffer per warp that is written out with one atomic reservation and
// coalesced stores.
constexpr int kWarpBuf = 512;  // buffered pairs per warp (one leaf visit adds at most 512)

__device__ __forceinline__ void warp_buf_flush(int2* bij, float* bd, int& nb,
                                               unsigned long long* cursor, int64_t cap,
                                               int32_t* pi, int32_t* pj, float* pd) {
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 0 && nb) base = atomicAdd(cursor, (unsigned long long)nb);
    base = __shfl_sync(0xffffffffu, base, 0);
    if ((int64_t)(base + (unsigned long long)nb) <= cap) {
        // the whole run fits: 32-bit offsets from the run's first slot
        int32_t* __restrict__ qi = pi + base;
        int32_t* __restrict__ qj = pj + base;
        float* __restrict__ qd = pd + base;
        for (int k = lane; k < nb; k += 32) {
            const int2 ij = bij[k];
            qi[k] = ij.x;
            qj[k] = ij.y;
            qd[k] = __fsqrt_rn(bd[k]);
        }
    } else {
        for (int k = lane; k < nb; k += 32) {
            const unsigned long long w = base + (unsigned long long)k;
            if ((int64_t)w < cap) {
                const int2 ij = bij[k];
                pi[w] = ij.x;
                pj[w] = ij.y;
                pd[w] = __fsqrt_rn(bd[k]);
            }
        }
    }
    __syncwarp();
    nb = 0;
}

// Appends this lane's hits (bit k of mask = pair (ia[k / 4], ib[k % 4]) at
// squared distance d2[k], the value the test compared) to the warp's buffer
// in bit-major order: for each k, the lanes holding bit k take consecutive
// slots, so every store of the warp is contiguous (no shared-memory bank
// conflicts).  The buffer holds squared distances; the flush writes their
// square roots, every lane of the flush taking one.
__device__ __forceinline__ void warp_emit16(unsigned mask, const float (&d2)[16],
                                            const int32_t (&ia)[4], const int32_t (&ib)[4],
                                            int2* bij, float* bd, int& nb,
                                            unsigned long long* cursor, int64_t cap, int32_t* pi,
                                            int32_t* pj, float* pd) {
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const unsigned total = __reduce_add_sync(0xffffffffu, (unsigned)__popc(mask));
    if (total == 0) return;
    if (nb + (int)total > kWarpBuf) warp_buf_flush(bij, bd, nb, cursor, cap, pi, pj, pd);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const bool hit = (mask >> k) & 1u;
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int at = nb + __popc(bal & below);
            bij[at] = make_int2(ia[k >> 2], ib[k & 3]);
            bd[at] = d2[k];
        }
        nb += __popc(bal);
    }
    __syncwarp();
}

// The 16 tests of leaf pair (a, b) (a == b: the six pairs inside the leaf):
// squared distances and the hit mask.
__device__ __forceinline__ unsigned leaf_tests16(const float4 (&qa)[4], const float4 (&tb)[4],
                                                 bool self, float r2, float (&d2)[16]) {
    unsigned mask = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int i = k >> 2, j = k & 3;
        d2[k] = dist2_ref(qa[i].x, qa[i].y, qa[i].z, tb[j].x, tb[j].y, tb[j].z);
        if ((!self || j > i) && d2[k] < r2) mask |= 1u << k;
    }
    return mask;
}

__global__ void __launch_bounds__(128, 6)
    k_leaf_warp4(const float4* __restrict__ keys, const float4* __restrict__ pos, int32_t nL,
                 float r, float r2, unsigned long long* cursor, int64_t cap, int32_t* pi,
                 int32_t* pj, float* pd, int32_t* err) {
    constexpr int APL = 4;
    const float r2g = r * r * 1.0001f;
    __shared__ int2 sbij[4][kWarpBuf];
    __shared__ float sbd[4][kWarpBuf];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int32_t q0 = (int32_t)((blockIdx.x * 4 + w) * 32) + 1;
    if (q0 > nL) return;  // whole warp
    int2* bij = sbij[w];
    float* bd = sbd[w];
    const int32_t q = q0 + lane;
    const bool valid = q <= nL;
    Node ql;
    float4 qa[APL];
    if (valid) {
        ql = load_node(keys, q);
        const int64_t A = (int64_t)(q - 1) * APL;
#pragma unroll
        for (int i = 0; i < APL; ++i) qa[i] = __ldg(&pos[A + i]);
    } else {
        ql.mnx = ql.mny = ql.mnz = INFINITY;
        ql.mxx = ql.mxy = ql.mxz = -INFINITY;
        ql.left = ql.skip = 0;
#pragma unroll
        for (int i = 0; i < APL; ++i) qa[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const float slack = valid ? leaf_slack(ql) : 0.0f;
    int nb = 0;
    int32_t ia[APL];
#pragma unroll
    for (int i = 0; i < APL; ++i) ia[i] = __float_as_int(qa[i].w);
    {
        // intra-leaf pairs (a before b in the leaf)
        float d2[16];
        unsigned mask = leaf_tests16(qa, qa, true, r2, d2);
        if (!valid) mask = 0;
        warp_emit16(mask, d2, ia, ia, bij, bd, nb, cursor, cap, pi, pj, pd);
    }
    // the warp's union box (invalid lanes contribute the empty box)
    Node un = ql;
    for (int sh = 16; sh > 0; sh >>= 1) {
        un.mnx = fminf(un.mnx, __shfl_xor_sync(0xffffffffu, un.mnx, sh));
        un.mny = fminf(un.mny, __shfl_xor_sync(0xffffffffu, un.mny, sh));
        un.mnz = fminf(un.mnz, __shfl_xor_sync(0xffffffffu, un.mnz, sh));
        un.mxx = fmaxf(un.mxx, __shfl_xor_sync(0xffffffffu, un.mxx, sh));
        un.mxy = fmaxf(un.mxy, __shfl_xor_sync(0xffffffffu, un.mxy, sh));
        un.mxz = fmaxf(un.mxz, __shfl_xor_sync(0xffffffffu, un.mxz, sh));
    }
    int32_t t = __shfl_sync(0xffffffffu, ql.skip, 0);
    int32_t visits = 0;
    const int32_t nnodes = 2 * nL - 1;
    while (t != 0) {
        if (t < 1 || t > nnodes || ++visits > nnodes) {
            if (lane == 0) set_error(err, ND_ERR_INTERNAL, q0);
            break;
        }
        const Node nd_ = load_node(keys, t);
        if (overlap(un, nd_)) {
            if (nd_.left == 0) {
                unsigned mask = 0;
                float d2[16];
                int32_t ib[APL] = {0, 0, 0, 0};
                if (valid && t > q && overlap(ql, nd_) && leaf_gap_ok(ql, nd_, r, r2g, slack)) {
                    const int64_t B = (int64_t)(t - 1) * APL;
                    float4 tb[APL];
#pragma unroll
                    for (int j = 0; j < APL; ++j) tb[j] = __ldg(&pos[B + j]);
                    mask = leaf_tests16(qa, tb, false, r2, d2);
#pragma unroll
                    for (int j = 0; j < APL; ++j) ib[j] = __float_as_int(tb[j].w);
                }
                warp_emit16(mask, d2, ia, ib, bij, bd, nb, cursor, cap, pi, pj, pd);
                t = nd_.skip;
            } else {
                t = nd_.left;
            }
        } else {
            t = nd_.skip;
        }
    }
    warp_buf_flush(bij, bd, nb, cursor, cap, pi, pj, pd);
}

__global__ void __launch_bounds__(128)
    k_atom_count(const float4* __restrict__ keys, const float4* __restrict__ pos, int32_t n,
                 int32_t apl, float r2, int64_t* __restrict__ counts, int32_t* err) {
    int32_t qi = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (qi > n) return;
    SinkCount s;
    if (qi <= n - 1) atom_query(qi, keys, pos, apl, r2, 2 * (n / apl) - 1, err, s);
    counts[qi - 1] = s.n;
}

__global__ void __launch_bounds__(128)
    k_atom_write(const float4* __restrict__ keys, const float4* __restrict__ pos, int32_t n,
                 int32_t apl, float r2, const int64_t* __restrict__ offsets, int32_t* pi,
                 int32_t* pj, float* pd, int32_t* err) {
    int32_t qi = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (qi > n - 1) return;
    SinkWrite s{pi, pj, pd, offsets[qi - 1]};
    atom_query(qi, keys, pos, apl, r2, 2 * (n / apl) - 1, err, s);
}

// Two-phase form of the one-pass emission, for callers that allow scratch
// memory.  Broad phase: the candidate leaf pairs (q, t) -- t > q with
// overlapping boxes, and (q, q) for the pairs inside q -- are recorded through
// per-warp shared buffers; the work per visited leaf is one box test.  Narrow
// phase: one thread per candidate leaf pair runs the 4 x 4 distance tests and
// emits through the warp buffers of k_leaf_warp4.  The distance tests, most of
// the work, are then spread evenly over the GPU however dense the points are.
//
// The broad phase itself is split in two so that no walk is long: the union
// walk of a warp's 32 query leaves (as in k_leaf_warp4) stops at subtrees of
// at most kTaskLeaves leaves and records each overlapping one as a task
// (group, subtree root); a flat pool of warps then walks the tasks' subtrees.
// In a dense cluster one warp's union overlaps thousands of leaves; its walk
// becomes a few hundred steps plus many short walks on other warps.
constexpr int kLeafBuf = 256;    // candidate leaf pairs buffered per warp
constexpr int kTaskLeaves = 64;  // largest subtree recorded as one task

__device__ __forceinline__ void lp_flush(int2* buf, int& nb, unsigned long long* cursor, int64_t cap,
                                         int2* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 0 && nb) base = atomicAdd(cursor, (unsigned long long)nb);
    base = __shfl_sync(0xffffffffu, base, 0);
    for (int k = lane; k < nb; k += 32) {
        const unsigned long long w = base + (unsigned long long)k;
        if ((int64_t)w < cap) out[w] = buf[k];
    }
    __syncwarp();
    nb = 0;
}

__device__ __forceinline__ void lp_append(bool want, int32_t q, int32_t t, int2* buf, int& nb,
                                          unsigned long long* cursor, int64_t cap,
                                          int2* __restrict__ out) {
    const unsigned bal = __ballot_sync(0xffffffffu, want);
    if (!bal) return;
    const int total = __popc(bal);
    if (nb + total > kLeafBuf) lp_flush(buf, nb, cursor, cap, out);
    if (want) buf[nb + __popc(bal & ((1u << (threadIdx.x & 31)) - 1u))] = make_int2(q, t);
    __syncwarp();
    nb += total;
}

// The query group of a warp: leaves q0 .. q0 + 31 (lane's own leaf, empty box
// past nL) and the union of their boxes.
__device__ __forceinline__ void group_boxes(const float4* __restrict__ keys, int32_t nL,
                                            int32_t q, Node& ql, Node& un) {
    if (q <= nL) {
        ql = load_node(keys, q);
    } else {
        ql.mnx = ql.mny = ql.mnz = INFINITY;
        ql.mxx = ql.mxy = ql.mxz = -INFINITY;
        ql.left = ql.skip = 0;
    }
    un = ql;
    for (int sh = 16; sh > 0; sh >>= 1) {
        un.mnx = fminf(un.mnx, __shfl_xor_sync(0xffffffffu, un.mnx, sh));
        un.mny = fminf(un.mny, __shfl_xor_sync(0xffffffffu, un.mny, sh));
        un.mnz = fminf(un.mnz, __shfl_xor_sync(0xffffffffu, un.mnz, sh));
        un.mxx = fmaxf(un.mxx, __shfl_xor_sync(0xffffffffu, un.mxx, sh));
        un.mxy = fmaxf(un.mxy, __shfl_xor_sync(0xffffffffu, un.mxy, sh));
        un.mxz = fmaxf(un.mxz, __shfl_xor_sync(0xffffffffu, un.mxz, sh));
    }
}

// Broad phase, first half: one warp per group of 32 query leaves.  The pairs
// inside each leaf go to the candidate list; the union walk from the skip rope
// of the group's first leaf records (group, node) for every overlapping node
// of at most kTaskLeaves leaves instead of descending into it.  Tasks are
// warp-uniform: lane k holds the k-th pending one, 32 are written at a time.
__global__ void __launch_bounds__(128)
    k_leaf_tasks4(const float4* __restrict__ keys, const int2* __restrict__ ranges, int32_t nL,
                  unsigned long long* cursor, int64_t cap, int2* __restrict__ out,
                  unsigned long long* tcursor, int64_t tcap, int2* __restrict__ tasks,
                  int32_t* err) {
    __shared__ int2 sbuf[4][kLeafBuf];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int32_t g = (int32_t)(blockIdx.x * 4 + w);
    const int32_t q0 = g * 32 + 1;
    if (q0 > nL) return;  // whole warp
    int2* buf = sbuf[w];
    const int32_t q = q0 + lane;
    Node ql, un;
    group_boxes(keys, nL, q, ql, un);
    int nb = 0;
    lp_append(q <= nL, q, q, buf, nb, cursor, cap, out);  // pairs inside the leaf
    lp_flush(buf, nb, cursor, cap, out);
    int2 mine = make_int2(0, 0);
    int npend = 0;
    auto flush_tasks = [&]() {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(tcursor, (unsigned long long)npend);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (lane < npend && (int64_t)(base + lane) < tcap) tasks[base + lane] = mine;
        npend = 0;
    };
    int32_t t = __shfl_sync(0xffffffffu, ql.skip, 0);
    int32_t visits = 0;
    const int32_t nnodes = 2 * nL - 1;
    while (t != 0) {
        if (t < 1 || t > nnodes || ++visits > nnodes) {
            if (lane == 0) set_error(err, ND_ERR_INTERNAL, q0);
            break;
        }
        const Node nd_ = load_node(keys, t);
        int32_t size = 1;
        if (t > nL) {
            const int2 rg = __ldg(&ranges[t - nL - 1]);
            size = rg.y - rg.x + 1;
        }
        if (overlap(un, nd_)) {
            if (size <= kTaskLeaves) {
                if (lane == npend) mine = make_int2(g, t);
                if (++npend == 32) flush_tasks();
                t = nd_.skip;
            } else {
                t = nd_.left;
            }
        } else {
            t = nd_.skip;
        }
    }
    if (npend) flush_tasks();
}

// Broad phase, second half: warps stride over the tasks.  A task's subtree
// holds the leaves of one contiguous range (at most kTaskLeaves); the warp
// scans them in order, four node loads in flight at a time, and records
// (q, t) for the lanes whose own leaf q < t overlaps t (a leaf overlapping q
// overlaps every ancestor, so these are the candidates a walk pruning with
// the group's union box would find) and whose atoms can be within r at all
// (leaf_gap_ok: about 40 % of the overlapping leaves in dense clusters are
// not).
__global__ void __launch_bounds__(128)
    k_leaf_subwalk4(const float4* __restrict__ keys, const int2* __restrict__ ranges, int32_t nL,
                    float r, const unsigned long long* __restrict__ tcount, int64_t tcap,
                    const int2* __restrict__ tasks, unsigned long long* cursor, int64_t cap,
                    int2* __restrict__ out, int32_t* err) {
    const float r2g = r * r * 1.0001f;  // the gap test is a filter: the distance test decides
    __shared__ int2 sbuf[4][kLeafBuf];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int2* buf = sbuf[w];
    int nb = 0;
    const int64_t ntask = min((int64_t)*tcount, tcap);
    const int32_t nnodes = 2 * nL - 1;
    for (int64_t k = (int64_t)blockIdx.x * 4 + w; k < ntask; k += (int64_t)gridDim.x * 4) {
        const int2 tk = __ldg(&tasks[k]);
        const int32_t q0 = tk.x * 32 + 1;
        const int32_t q = q0 + lane;
        const bool valid = q <= nL;
        Node ql, un;
        group_boxes(keys, nL, q, ql, un);
        const int32_t root = tk.y;
        if (root < 1 || root > nnodes) {
            if (lane == 0) set_error(err, ND_ERR_INTERNAL, tk.x);
            continue;
        }
        int32_t la = root, lb = root;  // leaf range of the subtree
        if (root > nL) {
            const int2 rg = __ldg(&ranges[root - nL - 1]);
            la = rg.x;
            lb = rg.y;
        }
        if (la < 1 || lb > nL || lb - la + 1 > kTaskLeaves) {
            if (lane == 0) set_error(err, ND_ERR_INTERNAL, tk.x);
            continue;
        }
        const float slack = valid ? leaf_slack(ql) : 0.0f;
        // leaves after the group's first only (t > q for some lane)
        for (int32_t t0 = max(la, q0 + 1); t0 <= lb; t0 += 4) {
            Node nd4[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (t0 + u <= lb) nd4[u] = load_node(keys, t0 + u);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int32_t t = t0 + u;
                if (t > lb) break;  // warp-uniform
                const Node& b = nd4[u];
                const bool want =
                    valid && t > q && overlap(ql, b) && leaf_gap_ok(ql, b, r, r2g, slack);
                lp_append(want, q, t, buf, nb, cursor, cap, out);
            }
        }
    }
    lp_flush(buf, nb, cursor, cap, out);
}

__global__ void __launch_bounds__(256)
    k_leaf_narrow4(const int2* __restrict__ lp, int64_t nlp, const float4* __restrict__ pos,
                   float r2, unsigned long long* cursor, int64_t cap, int32_t* pi, int32_t* pj,
                   float* pd) {
    constexpr int APL = 4;
    __shared__ int2 sbij[8][kWarpBuf];
    __shared__ float sbd[8][kWarpBuf];
    const int w = threadIdx.x >> 5;
    int2* bij = sbij[w];
    float* bd = sbd[w];
    int nb = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // warp-uniform trip count: lanes past the end test nothing but join the ballots
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
         __any_sync(0xffffffffu, k < nlp); k += stride) {
        unsigned mask = 0;
        float d2[16];
        int32_t ia[APL] = {0, 0, 0, 0}, ib[APL] = {0, 0, 0, 0};
        if (k < nlp) {
            const int2 e = __ldg(&lp[k]);
            const int64_t A = (int64_t)(e.x - 1) * APL, B = (int64_t)(e.y - 1) * APL;
            float4 qa[APL], tb[APL];
#pragma unroll
            for (int i = 0; i < APL; ++i) qa[i] = __ldg(&pos[A + i]);
#pragma unroll
            for (int j = 0; j < APL; ++j) tb[j] = __ldg(&pos[B + j]);
            mask = leaf_tests16(qa, tb, e.x == e.y, r2, d2);
#pragma unroll
            for (int i = 0; i < APL; ++i) {
                ia[i] = __float_as_int(qa[i].w);
                ib[i] = __float_as_int(tb[i].w);
            }
        }
        warp_emit16(mask, d2, ia, ib, bij, bd, nb, cursor, cap, pi, pj, pd);
    }
    warp_buf_flush(bij, bd, nb, cursor, cap, pi, pj, pd);
}

// The pair criterion as a threshold on the Float32 squared distance d2:
// ND_CRIT_SQUARED: d2 < r^2 (leafneighbor_traverse, BVHTraverse.jl:1048), the
// threshold fl(r * r); ND_CRIT_SQRT: sqrt(d2) < r (simdneighbor_traverse,
// ext/NaiveSIMD.jl:529,589), the smallest float T with sqrtf(T) >= r -- the
// square root is correctly rounded, hence monotonic, so sqrt(d2) < r exactly
// when d2 < T.  The kernels compare d2 with the threshold either way.
float pair_threshold(float r, int32_t criterion) {
    float t = r * r;
    if (criterion != ND_CRIT_SQRT) return t;
    while (t > 0.0f && std::sqrt(std::nextafter(t, 0.0f)) >= r) t = std::nextafter(t, 0.0f);
    while (std::sqrt(t) < r) t = std::nextafter(t, INFINITY);
    return t;
}

nd_status emit_unordered(Ctx* c, const TreeBuffers& t, float r, float r2, int32_t* pi,
                         int32_t* pj, float* pd, int64_t capacity, int64_t* total) {
    if (t.apl != 4) return ND_ERR_ARG;
    nd_status st;
    if ((st = ensure(c, c->misc, 64))) return st;
    unsigned long long* cursor = (unsigned long long*)c->misc.p;
    unsigned long long tot = 0;
    cudaError_t e;
    if (c->no_alloc) {
        // no scratch for candidate pairs: the one-pass walk
        cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), c->stream);
        k_leaf_warp4<<<(unsigned)cdiv(t.nL, 128), 128, 0, c->stream>>>(
            t.keys, t.pos4, t.nL, r, r2, cursor, capacity, pi, pj, pd, c->d_err);
        c->launches++;
    } else {
        // broad phase: tasks, then the tasks' subtree walks; re-run with
        // larger buffers while either list overflowed
        if (!t.ranges) return ND_ERR_INTERNAL;
        unsigned long long* tcursor = cursor + 1;
        unsigned long long nlp = 0, ntask = 0;
        int nsm = 0, occ = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_leaf_subwalk4, 128, 0);
        const int64_t ngroups = cdiv(t.nL, 32);
        for (int attempt = 0;; ++attempt) {
            int64_t lcap = (int64_t)(c->leafpairs.bytes / sizeof(int2));
            if (lcap < 16 * (int64_t)t.nL) {
                if ((st = ensure(c, c->leafpairs, sizeof(int2) * 16 * (size_t)t.nL))) return st;
                lcap = 16 * (int64_t)t.nL;
            }
            int64_t tcap = (int64_t)(c->tasks.bytes / sizeof(int2));
            if (tcap < 16 * ngroups) {
                if ((st = ensure(c, c->tasks, sizeof(int2) * 16 * (size_t)ngroups))) return st;
                tcap = 16 * ngroups;
            }
            cudaMemsetAsync(cursor, 0, 2 * sizeof(unsigned long long), c->stream);
            k_leaf_tasks4<<<(unsigned)cdiv(t.nL, 128), 128, 0, c->stream>>>(
                t.keys, t.ranges, t.nL, cursor, lcap, (int2*)c->leafpairs.p, tcursor, tcap,
                (int2*)c->tasks.p, c->d_err);
            k_leaf_subwalk4<<<(unsigned)(nsm * std::max(occ, 1)), 128, 0, c->stream>>>(
                t.keys, t.ranges, t.nL, r, tcursor, tcap, (const int2*)c->tasks.p, cursor, lcap,
                (int2*)c->leafpairs.p, c->d_err);
            c->launches += 2;
            if ((st = check_launch(c, "leaf pairs (broad phase)"))) return st;
            unsigned long long h[2] = {0, 0};
            e = cudaMemcpyAsync(h, cursor, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "candidate leaf pairs");
            nlp = h[0];
            ntask = h[1];
            if ((int64_t)nlp <= lcap && (int64_t)ntask <= tcap) break;
            if (attempt == 2) {
                c->last_error = "candidate leaf pairs: buffers kept overflowing";
                return ND_ERR_INTERNAL;
            }
            if ((int64_t)ntask > tcap &&
                (st = ensure(c, c->tasks, sizeof(int2) * (size_t)(ntask + ntask / 4))))
                return st;
            if ((int64_t)nlp > lcap &&
                (st = ensure(c, c->leafpairs, sizeof(int2) * (size_t)(nlp + nlp / 4))))
                return st;
        }
        cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), c->stream);
        const int64_t blocks = std::min<int64_t>(cdiv((int64_t)nlp, 256), (int64_t)nsm * 32);
        if (nlp > 0) {
            k_leaf_narrow4<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, c->stream>>>(
                (const int2*)c->leafpairs.p, (int64_t)nlp, t.pos4, r2, cursor, capacity, pi, pj,
                pd);
            c->launches++;
        }
    }
    if ((st = check_launch(c, "leaf pairs (unordered)"))) return st;
    e = cudaMemcpyAsync(&tot, cursor, sizeof(tot), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "pair count");
    if ((st = sync_and_check(c, "leaf pairs (unordered)"))) return st;
    *total = (int64_t)tot;
    return ND_OK;
}

nd_status count_pairs(Ctx* c, const TreeBuffers& t, float r2, int kind, int64_t* total) {
    nd_status st;
    int64_t nq = (kind == 0) ? t.nL : t.n;
    if ((st = ensure(c, c->counts, sizeof(int64_t) * (size_t)(nq + 1)))) return st;
    if ((st = ensure(c, c->offsets, sizeof(int64_t) * (size_t)(nq + 2)))) return st;
    int64_t* counts = (int64_t*)c->counts.p;
    int64_t* offsets = (int64_t*)c->offsets.p;
    unsigned grid = (unsigned)cdiv(nq, 128);
    if (kind == 0) {
        if (t.apl == 4)
            k_leaf_count<4><<<grid, 128, 0, c->stream>>>(t.keys, t.pos4, t.nL, t.apl, r2, counts, c->d_err);
        else
            k_leaf_count<0><<<grid, 128, 0, c->stream>>>(t.keys, t.pos4, t.nL, t.apl, r2, counts, c->d_err);
    } else {
        k_atom_count<<<grid, 128, 0, c->stream>>>(t.keys, t.pos4, t.n, t.apl, r2, counts, c->d_err);
    }
    c->launches++;
    if ((st = check_launch(c, "pair count"))) return st;
    if ((st = scan_exclusive(c, counts, offsets, nq, offsets + nq))) return st;
    int64_t tot = 0;
    cudaError_t e = cudaMemcpyAsync(&tot, offsets + nq, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "pair total");
    if ((st = sync_and_check(c, "pair count"))) return st;
    *total = tot;
    return ND_OK;
}

nd_status write_pairs(Ctx* c, const TreeBuffers& t, float r2, int kind, int32_t* pi, int32_t* pj,
                      float* pd) {
    int64_t nq = (kind == 0) ? t.nL : t.n;
    const int64_t* offsets = (const int64_t*)c->offsets.p;
    unsigned grid = (unsigned)cdiv(nq, 128);
    if (kind == 0) {
        if (t.apl == 4)
            k_leaf_write<4><<<grid, 128, 0, c->stream>>>(t.keys, t.pos4, t.nL, t.apl, r2, offsets,
                                                        pi, pj, pd, c->d_err);
        else
            k_leaf_write<0><<<grid, 128, 0, c->stream>>>(t.keys, t.pos4, t.nL, t.apl, r2, offsets,
                                                        pi, pj, pd, c->d_err);
    } else {
        k_atom_write<<<grid, 128, 0, c->stream>>>(t.keys, t.pos4, t.n, t.apl, r2, offsets, pi, pj,
                                                  pd, c->d_err);
    }
    c->launches++;
    return check_launch(c, "pair write");
}

// ================================================================ pair hash

__global__ void k_pair_hash(const int32_t* __restrict__ pi, const int32_t* __restrict__ pj,
                            const float* __restrict__ pd, int64_t np,
                            unsigned long long* out) {
    uint64_t h0 = 0, h1 = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < np;
         k += (int64_t)gridDim.x * blockDim.x)
        pair_hash_one(pi[k], pj[k], pd[k], h0, h1);
    for (int s = 16; s > 0; s >>= 1) {
        h0 += __shfl_xor_sync(0xffffffffu, h0, s);
        h1 += __shfl_xor_sync(0xffffffffu, h1, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], (unsigned long long)h0);
        atomicAdd(&out[1], (unsigned long long)h1);
    }
}

nd_status pair_hash(Ctx* c, const int32_t* pi, const int32_t* pj, const float* pd, int64_t np,
                    uint64_t out[2]) {
    nd_status st = ensure(c, c->hash, 16);
    if (st) return st;
    cudaMemsetAsync(c->hash.p, 0, 16, c->stream);
    if (np > 0) {
        int blocks = (int)std::min<int64_t>(cdiv(np, 256), 152 * 16);
        k_pair_hash<<<blocks, 256, 0, c->stream>>>(pi, pj, pd, np, (unsigned long long*)c->hash.p);
        c->launches++;
    }
    cudaError_t e = cudaMemcpyAsync(out, c->hash.p, 16, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "hash copy");
    return sync_and_check(c, "pair hash");
}

}  // namespace nd
