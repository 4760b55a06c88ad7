// nd_md.cu -- device-resident molecular dynamics for sm_103a: the GPU form of
// simulate! (src/Simulator.jl:154-256) with the intended physics of
// force_lennardjones! / force_coulomb! / sum_forces! (src/Forces.jl) and
// kick-drift-kick velocity Verlet with boundary_reflect! walls
// (src/Simulator.jl:81-111).
//
// Layout in HBM (atoms are kept in tree order and re-sorted at every rebuild):
//   x[3][N], w[3][N]   FP64 positions and velocities, one array per component
//                      (two sets, ping-ponged by the reorder at each rebuild)
//   q[N], im[N]        FP64 charge and inverse mass
//   rec[2][N]          int4 pair-math record per atom: fixed-point position
//                      (int32 x, y, z in units of 1/S from the frame origin)
//                      and the charge's float bits (ping-ponged per step)
//   pos32[N]           float4 Float32 positions at the last rebuild (tree input)
//   ulist[B][ucap]     per block of 256 atoms: the sorted leaves that hold any
//                      neighbour of the block (the block's union), ucount[B]
//   llist[B][lcap][256] uint16 per-atom neighbour lists as indices into the
//                      block's union (slot-major inside the block), ncount[N]
// One MD step is ONE kernel: a block stages its union's records in shared
// memory, each thread sums its atom's pair forces over its own exact list (no
// atomics, deterministic), completes the pending half kick, kicks, drifts,
// reflects and writes the next record.  Velocities are stored at half steps
// between kernels (w = v_{n-1/2} after reflection).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "nd_md_engine.cuh"

namespace nd {

constexpr int kSmallTPA = 4;         // threads per atom of the step kernel for small systems
constexpr int kSizingFcap = 8192;    // BFS frontier entries per buffer in the sizing build
constexpr int kSizingUcap = 8192;    // union capacity of the sizing build
constexpr double kMinTunedSkin = 0.1;  // smallest skin the autotuner tries

// Scale of the wrap-around fixed-point grid: a listed pair is within
// r_c + skin at the build and its atoms move at most skin/2 each before the
// next refit, so its per-axis separation stays below r_c + 2 skin; a quarter
// of head-room on top.  At r_c = 2.5 and skin 0.4 the grid step is 2^-28.
static double md_scale(const nd_md_params& p) {
    const double span = 1.25 * (p.cutoff + 2.0 * std::max(p.skin, 0.0));
    return std::ldexp(1.0, (int)std::floor(std::log2(2147483648.0 / span)));
}

// Near-pair constants of a system with LJ sigma, epsilon and Coulomb constant
// kc at grid scale S.  The split
// keeps hi = x_fp with its low k bits cleared below 2^(k+10) in magnitude for
// separations up to 1.25 rnb, so the sum of the three squared hi parts is an
// exact float.
static NearK md_near(double sigma, double eps, double kc, double rc, double S) {
    NearK k{};
    const double rn = 1.3 * sigma, rnb = rn + 0.1;
    k.rn2u = (float)(rn * rn * S * S);
    const double sig2 = sigma * sigma * S * S;
    k.sig2lo = (float)(sig2 - (double)(float)sig2);
    const double e24 = 24.0 * eps * S, kcu = kc * S * S;
    k.e24lo = (float)(e24 - (double)(float)e24);
    k.kclo = (float)(kcu - (double)(float)kcu);
    const double rc2 = rc * rc * S * S;
    k.rc2lo = (float)(rc2 - (double)(float)rc2);
    k.rnb2 = (float)(rnb * rnb);
    int b = (int)std::ceil(std::log2(1.25 * rnb * S)) - 10;
    b = std::min(std::max(b, 0), 23);
    k.hmask = (int32_t)(~((1u << b) - 1u));
    return k;
}

// Range bound of |x_fp| (before the wrap) for a frame at scale S whose walls
// span ext: sc is the coarsest power-of-two scale at which the frame (the
// walls and 1/16 of the extent on each side) fits int32, and a coordinate is
// in range while (x - o) sc does.
static double md_frame_lim(double ext, double S) {
    const double range = ext * 1.125;
    const double sc = std::ldexp(1.0, (int)std::floor(std::log2(2147480000.0 / range)));
    return 2147480000.0 * (S / sc);
}



// Packed single precision (sm_100 and later): one instruction applies the
// operation to both halves of a 64-bit register pair, so two list entries
// share each instruction of the pair arithmetic.  The forces are held to a
// tolerance against FP64, not to the scalar form's bits: a packed sequence
// can end an ulp away from the scalar one (measured on distance tests).
__device__ __forceinline__ uint64_t pk2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(uint64_t v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// both halves negated (sign bits flipped)
__device__ __forceinline__ uint64_t neg2(uint64_t a) { return a ^ 0x8000000080000000ull; }
__device__ __forceinline__ uint64_t sp2(float a) { return pk2(a, a); }

// ------------------------------------------------------------- small kernels

__global__ void k_md_split_aos(const double* __restrict__ aos, int32_t n, double* x0, double* x1,
                               double* x2) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x0[i] = aos[3 * (int64_t)i];
    x1[i] = aos[3 * (int64_t)i + 1];
    x2[i] = aos[3 * (int64_t)i + 2];
}

__global__ void k_md_init_scalars(const double* __restrict__ q_in, const double* __restrict__ m_in,
                                  const int32_t* __restrict__ sid_in, int32_t n, double* q,
                                  double* im, int32_t* orig, int32_t* sid) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    q[i] = q_in ? q_in[i] : 0.0;
    im[i] = m_in ? 1.0 / m_in[i] : 1.0;
    orig[i] = i;
    if (sid) sid[i] = sid_in[i];
}

__global__ void k_md_pos32(const double* __restrict__ x0, const double* __restrict__ x1,
                           const double* __restrict__ x2, const int32_t* __restrict__ sid,
                           const SysRow* __restrict__ sys, int32_t n, float* __restrict__ xyz,
                           unsigned* counter) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (counter && i == 0) atomicAdd(counter, 1u);
    if (i >= n) return;
    double o0 = 0.0, o1 = 0.0, o2 = 0.0;
    if (sid) {
        const SysRow* r = sys + sid[i];
        o0 = r->off[0]; o1 = r->off[1]; o2 = r->off[2];
    }
    xyz[3 * (int64_t)i] = (float)(x0[i] + o0);
    xyz[3 * (int64_t)i + 1] = (float)(x1[i] + o1);
    xyz[3 * (int64_t)i + 2] = (float)(x2[i] + o2);
}


// Gather every per-atom array into the new (sorted) order; write the pair
// records and the Float32 positions of the tree.
__global__ void k_md_reorder(SetPtrs src, SetPtrs dst, const int32_t* __restrict__ perm,
                             const float* __restrict__ xyz32, int32_t n, Frame fr,
                             const SysRow* __restrict__ sys, float4* __restrict__ pos32,
                             int4* __restrict__ rec, uint2* __restrict__ recf,
                             int4* __restrict__ recb, int32_t* err) {
    int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int32_t o = perm[k];
    const SysRow* r = nullptr;
    if (src.sid) {
        const int32_t sv = src.sid[o];
        dst.sid[k] = sv;
        r = sys + sv;
    }
    int32_t f[3];
    uint32_t g[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double xv = src.x[d][o];
        dst.x[d][k] = xv;
        dst.w[d][k] = src.w[d][o];
        f[d] = to_fixed(xv, r ? r->o[d] : fr.o[d], r ? r->s : fr.s, r ? r->lim : fr.lim, err, k,
                        g[d]);
    }
    recf[k] = pack_fine(g[0], g[1], g[2]);
    double qv = src.q[o];
    dst.q[k] = qv;
    dst.im[k] = src.im[o];
    dst.orig[k] = src.orig[o];
    pos32[k] = make_float4(xyz32[3 * (int64_t)o], xyz32[3 * (int64_t)o + 1],
                           xyz32[3 * (int64_t)o + 2], __int_as_float(k));
    rec[k] = make_int4(f[0], f[1], f[2], __float_as_int((float)qv));
    recb[k] = rec[k];
}

// Copy a state set (after the gather into the scratch set, so the live set
// keeps its addresses and captured graphs stay valid).
__global__ void k_md_copy_set(SetPtrs src, SetPtrs dst, int32_t n) {
    int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dst.x[d][k] = src.x[d][k];
        dst.w[d][k] = src.w[d][k];
    }
    dst.q[k] = src.q[k];
    dst.im[k] = src.im[k];
    dst.orig[k] = src.orig[k];
    if (src.sid) dst.sid[k] = src.sid[k];
}

// Start of a rebuild window: re-sort on the schedule (every resort_every-th
// window) or when some list has passed 90% of its capacity since the last
// re-sort (the kept tree has loosened); refit otherwise.  ctl[3] counts
// windows, ctl[4] holds the capacity-pressure flag, ctl[5] the decision.
__global__ void k_md_window_begin(unsigned* ctl, int32_t resort_every,
                                  cudaGraphConditionalHandle h, int32_t use_cond) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const unsigned w = ctl[3];
    const unsigned need = (w % (unsigned)resort_every == 0u || ctl[4] != 0u) ? 1u : 0u;
    ctl[3] = w + 1u;
    if (need) ctl[4] = 0u;
    ctl[5] = need;
    if (use_cond) cudaGraphSetConditional(h, need);
}

// Leaf boxes (p -/+ h) of already sorted Float32 positions.
__global__ void k_md_leaf_boxes(const float4* __restrict__ pos, int32_t nL, int32_t apl, float h,
                                float4* __restrict__ keys) {
    int32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= nL) return;
    int64_t bird = (int64_t)leaf * apl;
    float4 p0 = pos[bird];
    float mn[3] = {__fsub_rn(p0.x, h), __fsub_rn(p0.y, h), __fsub_rn(p0.z, h)};
    float mx[3] = {__fadd_rn(p0.x, h), __fadd_rn(p0.y, h), __fadd_rn(p0.z, h)};
    for (int32_t a = 1; a < apl; ++a) {
        float4 p = pos[bird + a];
        mn[0] = jl_min(mn[0], __fsub_rn(p.x, h)); mx[0] = jl_max(mx[0], __fadd_rn(p.x, h));
        mn[1] = jl_min(mn[1], __fsub_rn(p.y, h)); mx[1] = jl_max(mx[1], __fadd_rn(p.y, h));
        mn[2] = jl_min(mn[2], __fsub_rn(p.z, h)); mx[2] = jl_max(mx[2], __fadd_rn(p.z, h));
    }
    keys[2 * (int64_t)leaf] = make_float4(mn[0], mn[1], mn[2], mx[0]);
    keys[2 * (int64_t)leaf + 1] = make_float4(mx[1], mx[2], __int_as_float(0), __int_as_float(0));
}

// ------------------------------------------------ block union (tree BFS)

__device__ __forceinline__ bool box_overlap(float qmnx, float qmny, float qmnz, float qmxx,
                                            float qmxy, float qmxz, const float4& a,
                                            const float4& b) {
    // aabb_overlap_test (BVHTraverse.jl:1094-1098) against a node stored as
    // (min.x, min.y, min.z, max.x), (max.y, max.z, left, skip)
    return (qmnx < a.w) & (qmxx > a.x) & (qmny < b.x) & (qmxy > a.y) & (qmnz < b.y) &
           (qmxz > a.z);
}

// Boxes of the blocks of kBlock atoms (the union of their leaves' key boxes,
// exact: min / max only) and of the super-blocks of 32 blocks, stored like
// tree nodes (min xyz, max x), (max y, max z, 0, 0): blocks at [0, nblocks),
// super-blocks after them.  One thread block of 32 warps per super-block,
// one warp per block.
__global__ void __launch_bounds__(1024)
    k_md_block_boxes(const float4* __restrict__ keys, int32_t nL, int32_t nblocks, int32_t lpb,
                     float4* __restrict__ bbox) {
    __shared__ float s_b[32][6];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int32_t b = blockIdx.x * 32 + w;
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (b < nblocks) {
        const int32_t l1 = min((b + 1) * lpb, nL);
        for (int32_t l = b * lpb + lane; l < l1; l += 32) {
            const float4 a = __ldg(&keys[2 * (int64_t)l]), c = __ldg(&keys[2 * (int64_t)l + 1]);
            mn[0] = fminf(mn[0], a.x); mn[1] = fminf(mn[1], a.y); mn[2] = fminf(mn[2], a.z);
            mx[0] = fmaxf(mx[0], a.w); mx[1] = fmaxf(mx[1], c.x); mx[2] = fmaxf(mx[2], c.y);
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d)
        for (int s = 16; s > 0; s >>= 1) {
            mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], s));
            mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], s));
        }
    if (lane == 0) {
        if (b < nblocks) {
            bbox[2 * (int64_t)b] = make_float4(mn[0], mn[1], mn[2], mx[0]);
            bbox[2 * (int64_t)b + 1] = make_float4(mx[1], mx[2], 0.f, 0.f);
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) { s_b[w][d] = mn[d]; s_b[w][3 + d] = mx[d]; }
    }
    __syncthreads();
    if (w == 0) {
        float v[6];
#pragma unroll
        for (int d = 0; d < 6; ++d) v[d] = s_b[lane][d];
#pragma unroll
        for (int d = 0; d < 3; ++d)
            for (int s = 16; s > 0; s >>= 1) {
                v[d] = fminf(v[d], __shfl_xor_sync(0xffffffffu, v[d], s));
                v[3 + d] = fmaxf(v[3 + d], __shfl_xor_sync(0xffffffffu, v[3 + d], s));
            }
        if (lane == 0) {
            const int64_t sb = nblocks + (int64_t)blockIdx.x;
            bbox[2 * sb] = make_float4(v[0], v[1], v[2], v[3]);
            bbox[2 * sb + 1] = make_float4(v[4], v[5], 0.f, 0.f);
        }
    }
}

// Order-keeping compaction over the whole thread block: threads with `keep`
// write `value` to out[base + rank], rank counted in thread order.  Returns
// the number kept (the same in every thread).  Every thread must call it.
__device__ __forceinline__ int32_t block_compact(bool keep, int32_t value, int32_t* out,
                                                 int32_t base, int32_t cap, int32_t* s_w) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) s_w[warp] = __popc(bal);
    __syncthreads();
    int32_t off = base, total = 0;
#pragma unroll
    for (int w = 0; w < kBlock / 32; ++w) {
        const int32_t c = s_w[w];
        off += w < warp ? c : 0;
        total += c;
    }
    if (keep) {
        const int32_t at = off + __popc(bal & ((1u << lane) - 1u));
        if (at < cap) out[at] = value;
    }
    __syncthreads();
    return total;
}

// One block per 256 atoms: every leaf whose box overlaps one of the block's
// eight warp boxes (their atoms -/+ hq) joins the block's union, sorted by
// leaf index so list order, and hence force summation order, is
// deterministic.  Two searches give the same union:
//  - blocks (tree == 0): the super-block boxes, then the boxes of the blocks
//    of overlapping super-blocks, are tested against the union of the warp
//    boxes (a leaf overlapping a warp box lies in a block and a super-block
//    whose boxes overlap that union); the leaves of the candidate blocks are
//    tested against the warp boxes.  Enumerating in index order at every
//    level leaves the union sorted.
//  - tree (tree == 1): the warp boxes are tested against the tree
//    breadth-first -- all 256 threads expand the current level together, a
//    node's children being (left, skip of left) in the rope layout -- and the
//    union is sorted (bitonic) afterwards.
// Shared memory: two buffers of fcap entries (BFS frontiers, or candidate
// super-blocks and blocks) and the union (upow2).
__global__ void __launch_bounds__(kBlock)
    k_md_block_union(const float4* __restrict__ keys, const float4* __restrict__ bbox,
                     int32_t nblocks, int32_t tree, const float4* __restrict__ pos,
                     const int32_t* __restrict__ sid,
                     int32_t n, int32_t nL, int32_t apl, float hq, float rl, int32_t fcap,
                     int32_t ucap, int32_t upow2, int32_t* __restrict__ ulist,
                     int32_t* __restrict__ ucount,
                     uint16_t* __restrict__ llist_leaf, int32_t* __restrict__ lcount_leaf,
                     int32_t lcap_leaf, int32_t* err, int32_t* diag, int32_t sizing,
                     unsigned* pressure) {
    extern __shared__ int32_t smem[];
    int32_t* fr[2] = {smem, smem + fcap};
    int32_t* su = smem + 2 * fcap;
    __shared__ int32_t s_cnt[2];
    __shared__ int32_t s_nu, s_nb;
    __shared__ int32_t s_w[kBlock / 32];
    __shared__ float s_ub[6];
    // query boxes (min xyz, max xyz): one per warp, two for a warp whose atoms
    // belong to two systems of a batched ensemble (lanes of lane 0's system,
    // and the rest)
    __shared__ float s_wb[2 * (kBlock / 32)][6];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t i = (int64_t)blockIdx.x * kBlock + tid;
    if (tid == 0) { s_cnt[0] = 1; s_cnt[1] = 0; s_nu = 0; s_nb = 0; fr[0][0] = (nL + 1) << 1; }
    __syncthreads();
    {
        const int64_t ii = i < n ? i : (int64_t)blockIdx.x * kBlock;
        const float4 p = pos[ii];
        bool mine = true;
        if (sid) {
            const int32_t sv = __ldg(&sid[ii]);
            mine = sv == __shfl_sync(0xffffffffu, sv, 0);
        }
        const bool split = !__all_sync(0xffffffffu, mine);
        for (int part = 0; part < (split ? 2 : 1); ++part) {
            const bool in = (part == 0) == mine;
            float mn[3] = {in ? p.x : INFINITY, in ? p.y : INFINITY, in ? p.z : INFINITY};
            float mx[3] = {in ? p.x : -INFINITY, in ? p.y : -INFINITY, in ? p.z : -INFINITY};
#pragma unroll
            for (int d = 0; d < 3; ++d)
                for (int s = 16; s > 0; s >>= 1) {
                    mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], s));
                    mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], s));
                }
            if (lane == 0) {
                const int b = atomicAdd(&s_nb, 1);
                for (int d = 0; d < 3; ++d) { s_wb[b][d] = mn[d] - hq; s_wb[b][3 + d] = mx[d] + hq; }
            }
        }
    }
    __syncthreads();
    const int nb = s_nb;
    int32_t nu;
    if (!tree) {
        if (tid < 6) {
            float v = tid < 3 ? INFINITY : -INFINITY;
            for (int w = 0; w < nb; ++w) v = tid < 3 ? fminf(v, s_wb[w][tid]) : fmaxf(v, s_wb[w][tid]);
            s_ub[tid] = v;
        }
        __syncthreads();
        const float u0 = s_ub[0], u1 = s_ub[1], u2 = s_ub[2], u3 = s_ub[3], u4 = s_ub[4],
                    u5 = s_ub[5];
        int32_t* csb = fr[0];
        int32_t* cb = fr[1];
        const int32_t nsb = (nblocks + 31) >> 5;
        int32_t ncs = 0;
        for (int32_t base = 0; base < nsb; base += kBlock) {
            const int32_t s = base + tid;
            const bool keep = s < nsb && box_overlap(u0, u1, u2, u3, u4, u5,
                                                     __ldg(&bbox[2 * ((int64_t)nblocks + s)]),
                                                     __ldg(&bbox[2 * ((int64_t)nblocks + s) + 1]));
            ncs += block_compact(keep, s, csb, ncs, fcap, s_w);
        }
        int32_t ncb = 0;
        const int32_t ks = min(ncs, fcap) * 32;
        for (int32_t base = 0; base < ks; base += kBlock) {
            const int32_t k = base + tid;
            const int32_t b = k < ks ? csb[k >> 5] * 32 + (k & 31) : nblocks;
            const bool keep = b < nblocks && box_overlap(u0, u1, u2, u3, u4, u5,
                                                         __ldg(&bbox[2 * (int64_t)b]),
                                                         __ldg(&bbox[2 * (int64_t)b + 1]));
            ncb += block_compact(keep, b, cb, ncb, fcap, s_w);
        }
        if (tid == 0) {
            const int32_t mc = max(ncs, ncb);
            atomicMax(&diag[4], mc);
            if (pressure && 10 * mc > 9 * fcap) atomicOr(pressure, 1u);
            if (mc > fcap && !sizing) set_error(err, ND_ERR_OVERFLOW, (int32_t)blockIdx.x);
        }
        const int32_t lpb = kBlock / apl, lsh = __ffs(lpb) - 1;  // leaves per block (2^lsh)
        const int32_t kl = min(ncb, fcap) << lsh;
        nu = 0;
        for (int32_t base = 0; base < kl; base += kBlock) {
            const int32_t k = base + tid;
            const int32_t leaf = k < kl ? (cb[k >> lsh] << lsh) + (k & (lpb - 1)) : nL;
            bool hit = false;
            if (leaf < nL) {
                const float4 a = __ldg(&keys[2 * (int64_t)leaf]);
                const float4 b = __ldg(&keys[2 * (int64_t)leaf + 1]);
                for (int w = 0; w < nb && !hit; ++w)
                    hit = box_overlap(s_wb[w][0], s_wb[w][1], s_wb[w][2], s_wb[w][3], s_wb[w][4],
                                      s_wb[w][5], a, b);
            }
            nu += block_compact(hit, leaf, su, nu, upow2, s_w);
        }
    } else {
        int cur = 0;
        for (int level = 0; level < 256; ++level) {
            const int32_t nf = min(s_cnt[cur], fcap);
            if (nf == 0) break;
            for (int32_t k = tid; k < nf; k += kBlock) {
                const int32_t e = fr[cur][k];
                const int32_t t = e >> 1;
                if (t < 1 || t > 2 * nL - 1) { set_error(err, ND_ERR_INTERNAL, (int32_t)blockIdx.x); continue; }
                const float4 a = __ldg(&keys[2 * (int64_t)(t - 1)]);
                const float4 b = __ldg(&keys[2 * (int64_t)(t - 1) + 1]);
                const int32_t left = __float_as_int(b.z), skip = __float_as_int(b.w);
                if (e & 1) {  // a left child: its skip rope is its right sibling
                    int32_t slot = atomicAdd(&s_cnt[cur ^ 1], 1);
                    if (slot < fcap) fr[cur ^ 1][slot] = skip << 1;
                }
                bool hit = false;
                for (int w = 0; w < nb && !hit; ++w)
                    hit = box_overlap(s_wb[w][0], s_wb[w][1], s_wb[w][2], s_wb[w][3], s_wb[w][4],
                                      s_wb[w][5], a, b);
                if (hit) {
                    if (left == 0) {
                        int32_t slot = atomicAdd(&s_nu, 1);
                        if (slot < upow2) su[slot] = t - 1;
                    } else {
                        int32_t slot = atomicAdd(&s_cnt[cur ^ 1], 1);
                        if (slot < fcap) fr[cur ^ 1][slot] = (left << 1) | 1;
                    }
                }
            }
            __syncthreads();
            if (tid == 0) {
                atomicMax(&diag[4], s_cnt[cur ^ 1]);
                if (s_cnt[cur ^ 1] > fcap && !sizing) set_error(err, ND_ERR_INTERNAL, (int32_t)blockIdx.x);
                s_cnt[cur] = 0;
            }
            cur ^= 1;
            __syncthreads();
        }
        nu = s_nu;
    }
    if (tid == 0) { atomicMax(&diag[0], nu); atomicAdd(&diag[3], nu); }
    if (tid == 0 && pressure && 10 * (int64_t)nu > 9 * (int64_t)ucap) atomicOr(pressure, 1u);
    if (nu > ucap) {
        if (tid == 0 && !sizing) set_error(err, ND_ERR_OVERFLOW, (int32_t)blockIdx.x);
        if (tid == 0) ucount[blockIdx.x] = 0;
        for (int32_t k = tid; k < kBlock / apl; k += kBlock) {
            const int64_t leaf = (int64_t)blockIdx.x * (kBlock / apl) + k;
            if (leaf < nL) lcount_leaf[leaf] = 0;
        }
        return;
    }
    // bitonic sort of the union (padded to a power of two); the block search
    // enumerates it in order
    if (tree) {
        int32_t p2 = 1;
        while (p2 < nu) p2 <<= 1;
        for (int32_t k = nu + tid; k < p2; k += kBlock) su[k] = INT32_MAX;
        __syncthreads();
        for (int32_t size = 2; size <= p2; size <<= 1) {
            for (int32_t stride = size >> 1; stride > 0; stride >>= 1) {
                for (int32_t k = tid; k < p2 / 2; k += kBlock) {
                    int32_t lo = 2 * k - (k & (stride - 1));
                    int32_t hi = lo + stride;
                    bool up = ((lo & size) == 0);
                    int32_t a = su[lo], b = su[hi];
                    if ((a > b) == up) { su[lo] = b; su[hi] = a; }
                }
                __syncthreads();
            }
        }
    }
    int32_t* dst = ulist + (int64_t)blockIdx.x * ucap;
    for (int32_t k = tid; k < nu; k += kBlock) dst[k] = su[k];
    if (tid == 0) ucount[blockIdx.x] = nu;
    // Per-leaf candidate lists: for each of its leaves a warp keeps the union
    // positions whose atoms can be within r_list of that leaf's atoms at all,
    // ballot-compacted in union order: leaf boxes are atom boxes -/+ r_list/2,
    // and the Euclidean gap of the atom boxes (sqrt of the summed squared
    // per-axis gaps) must be below r_list -- a tighter test than the overlap of
    // the leaf boxes (the leaf-leaf test of leafneighbor_traverse,
    // BVHTraverse.jl:1282), which it implies, as it also drops the candidates
    // diagonally off the leaf.  A lane loads one union box per chunk and tests
    // it against the box of up to eight own leaves together; the union leaves
    // that pass are queued (per warp, in union order) and tested 32 at a time
    // against each of those own leaves.  The own boxes are widened by a few
    // ulps so no pair is lost to rounding; the atom distance test decides.
    __shared__ float s_own[kBlock / 32][8][6];
    __shared__ int32_t s_qu[kBlock / 32][64];    // per-warp queue: union index
    __shared__ float s_qb[kBlock / 32][6][64];   // and its key box
    const unsigned below = (1u << lane) - 1u;
    const float rl2g = rl * rl * 1.0002f;
    const int32_t leaves_per_warp = 32 / apl;
    const int64_t first_own = ((int64_t)blockIdx.x * kBlock + warp * 32) / apl;
    for (int32_t k0 = 0; k0 < leaves_per_warp; k0 += 8) {
        const int32_t nown = min(8, leaves_per_warp - k0);
        if (lane < nown) {
            const int64_t own = first_own + k0 + lane;
            float4 oa = make_float4(1.f, 1.f, 1.f, -1.f), ob = make_float4(-1.f, -1.f, 0.f, 0.f);
            if (own < nL) { oa = __ldg(&keys[2 * own]); ob = __ldg(&keys[2 * own + 1]); }
            s_own[warp][lane][0] = oa.x - 1e-5f * fabsf(oa.x) - 1e-6f;
            s_own[warp][lane][1] = oa.y - 1e-5f * fabsf(oa.y) - 1e-6f;
            s_own[warp][lane][2] = oa.z - 1e-5f * fabsf(oa.z) - 1e-6f;
            s_own[warp][lane][3] = oa.w + 1e-5f * fabsf(oa.w) + 1e-6f;
            s_own[warp][lane][4] = ob.x + 1e-5f * fabsf(ob.x) + 1e-6f;
            s_own[warp][lane][5] = ob.y + 1e-5f * fabsf(ob.y) + 1e-6f;
        }
        __syncwarp();
        // the group box: the union of these own boxes; a union leaf whose
        // atoms cannot come within r_list of it is dropped for all of them
        float gb[6];
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            float v = lane < nown ? s_own[warp][lane][d] : (d < 3 ? INFINITY : -INFINITY);
#pragma unroll
            for (int sh = 16; sh > 0; sh >>= 1) {
                const float w = __shfl_xor_sync(0xffffffffu, v, sh);
                v = d < 3 ? fminf(v, w) : fmaxf(v, w);
            }
            gb[d] = v;
        }
        // Euclidean gap test of key box (a, b) against box o (6 floats): the
        // per-axis gap of the atom boxes is the key-box gap + r_list, and a
        // Euclidean gap below r_list implies overlapping key boxes
        auto near_box = [&](const float* o, const float4& a, const float4& b) {
            const float gx = fmaxf(fmaxf(o[0] - a.w, a.x - o[3]) + rl, 0.0f);
            const float gy = fmaxf(fmaxf(o[1] - b.x, a.y - o[4]) + rl, 0.0f);
            const float gz = fmaxf(fmaxf(o[2] - b.y, a.z - o[5]) + rl, 0.0f);
            return gx * gx + gy * gy + gz * gz < rl2g;
        };
        int32_t lc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        // the passing union leaves go through a per-warp queue (in union
        // order), tested against the own leaves 32 at a time
        auto test_queue = [&](int32_t cnt) {
            const bool live = lane < cnt;
            const int32_t u = live ? s_qu[warp][lane] : 0;
            const float4 a = make_float4(s_qb[warp][0][lane], s_qb[warp][1][lane],
                                         s_qb[warp][2][lane], s_qb[warp][3][lane]);
            const float4 b = make_float4(s_qb[warp][4][lane], s_qb[warp][5][lane], 0.f, 0.f);
#pragma unroll
            for (int kl = 0; kl < 8; ++kl) {
                if (kl >= nown) break;
                const bool hit = live && near_box(s_own[warp][kl], a, b);
                const unsigned m = __ballot_sync(0xffffffffu, hit);
                const int32_t pos = lc[kl] + __popc(m & below);
                if (hit && pos < lcap_leaf)
                    llist_leaf[(first_own + k0 + kl) * lcap_leaf + pos] = (uint16_t)u;
                lc[kl] += __popc(m);
            }
        };
        int32_t qn = 0;
        for (int32_t base = 0; base < nu; base += 32) {
            const int32_t u = base + lane;
            float4 a = make_float4(1.f, 1.f, 1.f, -1.f), b = make_float4(-1.f, -1.f, 0.f, 0.f);
            if (u < nu) {
                const int32_t leaf = su[u];
                a = __ldg(&keys[2 * (int64_t)leaf]);
                b = __ldg(&keys[2 * (int64_t)leaf + 1]);
            }
            const bool pass = u < nu && near_box(gb, a, b);
            const unsigned m = __ballot_sync(0xffffffffu, pass);
            if (pass) {
                const int32_t at = qn + __popc(m & below);  // < 64: qn < 32 here
                s_qu[warp][at] = u;
                s_qb[warp][0][at] = a.x; s_qb[warp][1][at] = a.y; s_qb[warp][2][at] = a.z;
                s_qb[warp][3][at] = a.w; s_qb[warp][4][at] = b.x; s_qb[warp][5][at] = b.y;
            }
            qn += __popc(m);
            __syncwarp();
            if (qn >= 32) {
                test_queue(32);
                __syncwarp();
                // the rest to the front (sources at 32.., destinations below)
                if (lane < qn - 32) {
                    s_qu[warp][lane] = s_qu[warp][32 + lane];
#pragma unroll
                    for (int d = 0; d < 6; ++d) s_qb[warp][d][lane] = s_qb[warp][d][32 + lane];
                }
                qn -= 32;
                __syncwarp();
            }
        }
        if (qn > 0) test_queue(qn);
        if (lane < nown) {
            int32_t mine = 0;
#pragma unroll
            for (int kl = 0; kl < 8; ++kl)
                if (kl == lane) mine = lc[kl];
            const int64_t own = first_own + k0 + lane;
            if (own < nL) {
                lcount_leaf[own] = min(mine, lcap_leaf);
                atomicMax(&diag[2], mine);
                if (pressure && 10 * mine > 9 * lcap_leaf) atomicOr(pressure, 1u);
                if (mine > lcap_leaf && !sizing) set_error(err, ND_ERR_OVERFLOW, (int32_t)own);
            }
        }
        __syncwarp();
    }
}

// Exact per-atom lists inside the block's union: the union's Float32
// positions are staged in shared memory (up to smpos entries; the rest are read
// from L2), then the APL lanes of a leaf walk that leaf's candidate list
// together, each testing its own atom against the candidate leaf's atoms with
// the reference distance (Float32, d^2 < r_list^2) and storing union indices
// as uint16: entries closer than the near bound (rnb2, or the atom's system's)
// from slot 0 upwards, the others from slot lcap - 1 downwards.  pos.w holds
// the atom's sorted index (excludes the atom itself).  (Two atoms per packed
// f32x2 instruction measured slower here, and its sums are not always the
// scalar operations' bits: one pair of the 512-system ensemble came out 1 ulp
// above r_list^2.)
template <int APL>
__global__ void __launch_bounds__(kBlock)
    k_md_block_lists(const float4* __restrict__ pos, int32_t n, float rl2, float rnb2,
                     const int32_t* __restrict__ sid, const SysRow* __restrict__ sys,
                     int32_t ucap,
                     int32_t smpos, const int32_t* __restrict__ ulist,
                     const int32_t* __restrict__ ucount, const uint16_t* __restrict__ llist_leaf,
                     const int32_t* __restrict__ lcount_leaf, int32_t lcap_leaf, int32_t lcap,
                     uint16_t* __restrict__ llist, int32_t* __restrict__ ncount, int32_t* err,
                     int32_t* diag, int32_t sizing, unsigned* pressure) {
    extern __shared__ float4 spos[];
    const int tid = threadIdx.x;
    const int32_t* __restrict__ U = ulist + (int64_t)blockIdx.x * ucap;
    {
        // four positions per thread in flight: their leaf indices, then the
        // positions
        const int32_t nu = min(__ldg(&ucount[blockIdx.x]), ucap);
        const int32_t m = min(nu * APL, smpos);
        for (int32_t k = tid; k < m; k += 4 * kBlock) {
            int32_t lf[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int32_t kk = k + j * kBlock;
                lf[j] = kk < m ? __ldg(&U[kk / APL]) : 0;
            }
            float4 r[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int32_t kk = k + j * kBlock;
                if (kk < m) r[j] = __ldg(&pos[(int64_t)lf[j] * APL + (kk % APL)]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int32_t kk = k + j * kBlock;
                if (kk < m) spos[kk] = r[j];
            }
        }
    }
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * kBlock + tid;
    const bool valid = i < n;
    const int64_t own = (valid ? i : (int64_t)blockIdx.x * kBlock) / APL;
    const float4 p = __ldg(&pos[valid ? i : (int64_t)blockIdx.x * kBlock]);
    const int32_t nc = valid ? min(__ldg(&lcount_leaf[own]), lcap_leaf) : 0;
    // candidate entries eight at a time (a leaf's list starts on a 16-byte
    // boundary: lcap_leaf is a multiple of 8), the next eight loaded while the
    // current ones are tested
    const uint4* __restrict__ C = reinterpret_cast<const uint4*>(llist_leaf + own * lcap_leaf);
    uint16_t* __restrict__ L = llist + (int64_t)blockIdx.x * lcap * kBlock + tid;
    const int32_t self = (int32_t)i;
    const float nb2 = sid ? __ldg(&sys[__ldg(&sid[valid ? i : (int64_t)blockIdx.x * kBlock])].nk.rnb2)
                          : rnb2;
    int32_t cnt = 0, nn = 0, nf = 0;  // all hits; near and other entries stored
    // compiled twice: for a block whose whole union is staged (block-uniform)
    // the positions come from shared memory with no test
    auto walk = [&](auto staged) {
        constexpr bool ALL = decltype(staged)::value;
        uint4 nxt = nc > 0 ? __ldg(&C[0]) : make_uint4(0u, 0u, 0u, 0u);
        for (int32_t k0 = 0; k0 < nc; k0 += 8) {
            const uint4 cur = nxt;
            if (k0 + 8 < nc) nxt = __ldg(&C[(k0 >> 3) + 1]);
            const uint32_t cw[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                if (k0 + h >= nc) break;
                const int32_t u = (int32_t)((cw[h >> 1] >> (16 * (h & 1))) & 0xffffu);
                float4 q[APL];
                if (ALL || (u + 1) * APL <= smpos) {
#pragma unroll
                    for (int e = 0; e < APL; ++e) q[e] = spos[u * APL + e];
                } else {
                    const int64_t base = (int64_t)__ldg(&U[u]) * APL;
#pragma unroll
                    for (int e = 0; e < APL; ++e) q[e] = __ldg(&pos[base + e]);
                }
#pragma unroll
                for (int e = 0; e < APL; ++e) {
                    // branch-free: a predicated store to the near or the far end
                    const float d2 = dist2_ref(p.x, p.y, p.z, q[e].x, q[e].y, q[e].z);
                    const bool hit = d2 < rl2 && __float_as_int(q[e].w) != self;
                    const bool put = hit && cnt < lcap;
                    const bool near = d2 < nb2;
                    const int32_t slot = near ? nn : lcap - 1 - nf;
                    if (put) L[slot * kBlock] = (uint16_t)(u * APL + e);
                    nn += (put && near) ? 1 : 0;
                    nf += (put && !near) ? 1 : 0;
                    cnt += hit ? 1 : 0;
                }
            }
        }
    };
    if (min(__ldg(&ucount[blockIdx.x]), ucap) * APL <= smpos)
        walk(std::true_type{});
    else
        walk(std::false_type{});
    if (!valid) return;
    ncount[i] = nn | (nf << 16);
    if (cnt > lcap && !sizing) set_error(err, ND_ERR_OVERFLOW, (int32_t)i);
    atomicMax(&diag[1], cnt);
    if (pressure && 10 * cnt > 9 * lcap) atomicOr(pressure, 1u);
}

// Refit: positions changed, order and tree topology kept.  Float32 positions
// and pair records (and the build records of the skin check) from the FP64
// state in its current order.
__global__ void k_md_refit_pos(SetPtrs st, int32_t n, Frame fr, const SysRow* __restrict__ sys,
                               float4* __restrict__ pos32, int4* __restrict__ rec,
                               uint2* __restrict__ recf, int4* __restrict__ recb, int32_t* err,
                               unsigned* counter) {
    int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (counter && k == 0) atomicAdd(counter, 1u);
    if (k >= n) return;
    const SysRow* r = st.sid ? sys + st.sid[k] : nullptr;
    int32_t f[3];
    uint32_t g[3];
    float xf[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double xv = st.x[d][k];
        xf[d] = (float)(r ? xv + r->off[d] : xv);
        f[d] = to_fixed(xv, r ? r->o[d] : fr.o[d], r ? r->s : fr.s, r ? r->lim : fr.lim, err, k,
                        g[d]);
    }
    recf[k] = pack_fine(g[0], g[1], g[2]);
    pos32[k] = make_float4(xf[0], xf[1], xf[2], __int_as_float(k));
    const int4 rv = make_int4(f[0], f[1], f[2], __float_as_int((float)st.q[k]));
    rec[k] = rv;
    recb[k] = rv;
}

// ------------------------------------------------------------- step kernel


// Pair constants of one system in fixed-point units.
struct PairK {
    float rc2u, sig2u, eps24u, eps4, kcu, kceu;
    float rn2u, sig2lo, e24lo, kclo, rc2lo;
    int32_t hmask;
    // half-width of the band around rc2u inside which a single-precision r^2
    // (a few ulps off) cannot decide the cutoff: 2^-19 rc2u
    __device__ __forceinline__ float band() const { return rc2u * 1.9073486328125e-06f; }
};

// Low part of a separation split: the value in [0, 2^23) as a float, exact,
// by placing it in the mantissa of 2^23.
__device__ __forceinline__ float lo_part(int32_t v) {
    return __fsub_rn(__int_as_float(0x4B000000 | v), 8388608.0f);
}

// A force as three two-float sums (hi + lo per component).
struct DF3 {
    float xh, xl, yh, yl, zh, zl;
};

// (h, l) += (t, tl): TwoSum of the high parts (Knuth), low parts added.
__device__ __forceinline__ void df_acc(float& h, float& l, float t, float tl) {
    const float s = __fadd_rn(h, t);
    const float bb = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(t, bb));
    h = s;
    l = __fadd_rn(l, __fadd_rn(e, tl));
}

// Fine-grid difference of one coordinate (16-bit fields), in coarse units.
__device__ __forceinline__ float fine_diff(uint32_t a, uint32_t b, int sh) {
    const int32_t d = (int32_t)((a >> sh) & 0xffffu) - (int32_t)((b >> sh) & 0xffffu);
    return __fmul_rn(__int2float_rn(d), 1.52587890625e-05f);  // 2^-16, exact
}

// Near pair (i, j), separation below 1.3 sigma: the pair term in two-float
// arithmetic (each quantity a float pair hi + lo carrying about 44 bits), so
// that an atom whose large near terms cancel keeps its small net force to
// FP64-like accuracy.  The steep part of the potential amplifies a relative
// error in r^2 about 30-fold near its minimum (where 2 s6 - 1 cancels) and
// the terms reach hundreds at r < sigma, so every step carries its residual:
//  * separation: the coarse integer difference splits exactly into hi (low k
//    bits cleared, at most 11 significant bits) + lo (< 2^k); the fine-grid
//    difference (16 more bits) is added; sum hi^2 is an exact float, the rest
//    of r^2 and the rounding of the sum are kept in r2lo (Fast2Sum);
//  * 1/r^2 = ir2 (1 + eta): eta from the exact residual 1 - r2 ir2 (FMA) and
//    r2lo, so the approximate reciprocal square root needs no Newton step;
//  * every product with its FMA residual (Dekker), 2 s6 - 1 by TwoSum;
//  * the term's three components added to two-float sums (df_acc).
// Explicitly rounded operations (__f*_rn) keep the compiler from contracting
// a product whose residual is taken separately.
template <bool COUL, bool ENERGY>
__device__ __forceinline__ void accum_near(const int4& ri, const int4& rj, const uint2& fi,
                                           const uint2& fj, const PairK& a, DF3& acc, double& ue) {
    const int32_t ix = idiff(ri.x, rj.x), iy = idiff(ri.y, rj.y), iz = idiff(ri.z, rj.z);
    const float hx = __int2float_rn(ix & a.hmask), lx = lo_part(ix & ~a.hmask);
    const float hy = __int2float_rn(iy & a.hmask), ly = lo_part(iy & ~a.hmask);
    const float hz = __int2float_rn(iz & a.hmask), lz = lo_part(iz & ~a.hmask);
    const float fx = fine_diff(fi.x, fj.x, 0), fy = fine_diff(fi.x, fj.x, 16),
                fz = fine_diff(fi.y, fj.y, 0);
    // separation as two floats per axis: d = dh + dl
    const float dxh = __fadd_rn(hx, lx), dyh = __fadd_rn(hy, ly), dzh = __fadd_rn(hz, lz);
    const float dxl = __fadd_rn(__fsub_rn(lx, __fsub_rn(dxh, hx)), fx);
    const float dyl = __fadd_rn(__fsub_rn(ly, __fsub_rn(dyh, hy)), fy);
    const float dzl = __fadd_rn(__fsub_rn(lz, __fsub_rn(dzh, hz)), fz);
    const float P = __fmaf_rn(hz, hz, __fmaf_rn(hy, hy, __fmul_rn(hx, hx)));  // exact
    const float t = __fmaf_rn(hx, lx, __fmaf_rn(hy, ly, __fmul_rn(hz, lz)));
    const float l2 = __fmaf_rn(lx, lx, __fmaf_rn(ly, ly, __fmul_rn(lz, lz)));
    const float u = __fmaf_rn(dxh, fx, __fmaf_rn(dyh, fy, __fmul_rn(dzh, fz)));
    const float cl = __fmaf_rn(2.0f, u, __fmaf_rn(2.0f, t, l2));
    const float r2 = __fadd_rn(P, cl);
    const float r2lo = __fsub_rn(cl, __fsub_rn(r2, P));
    // the cutoff on the two-float r^2 against the two-float r_c^2 (exact where
    // they are close: Sterbenz), so a pair at r_c is in or out as in FP64
    if (!(__fadd_rn(__fsub_rn(r2, a.rc2u), __fsub_rn(r2lo, a.rc2lo)) < 0.0f)) return;
    const float ir = rsqrtf(r2);
    const float ir2 = __fmul_rn(ir, ir);
    const float eta = __fmaf_rn(-r2lo, ir2, __fmaf_rn(-r2, ir2, 1.0f));
    const float ir2l = __fmul_rn(ir2, eta);
    // s2 = sigma^2 / r^2, s4, s6 as two floats
    const float s2 = __fmul_rn(a.sig2u, ir2);
    const float s2l = __fmaf_rn(a.sig2lo, ir2, __fmaf_rn(a.sig2u, ir2l, __fmaf_rn(a.sig2u, ir2, -s2)));
    const float s4 = __fmul_rn(s2, s2);
    const float s4l = __fmaf_rn(__fmul_rn(2.0f, s2), s2l, __fmaf_rn(s2, s2, -s4));
    const float s6 = __fmul_rn(s4, s2);
    const float s6l = __fmaf_rn(s4, s2l, __fmaf_rn(s4l, s2, __fmaf_rn(s4, s2, -s6)));
    // w = 2 s6 - 1
    const float a2 = __fmul_rn(2.0f, s6);
    const float wh = __fsub_rn(a2, 1.0f);
    const float wb = __fsub_rn(wh, a2);
    const float we = __fadd_rn(__fsub_rn(a2, __fsub_rn(wh, wb)), __fsub_rn(-1.0f, wb));
    const float wl = __fmaf_rn(2.0f, s6l, we);
    // LJ magnitude 24 eps / r^2 s6 (2 s6 - 1)
    const float p1 = __fmul_rn(ir2, s6);
    const float p1l = __fmaf_rn(ir2l, s6, __fmaf_rn(ir2, s6l, __fmaf_rn(ir2, s6, -p1)));
    const float p2 = __fmul_rn(p1, wh);
    const float p2l = __fmaf_rn(p1l, wh, __fmaf_rn(p1, wl, __fmaf_rn(p1, wh, -p2)));
    float fh = __fmul_rn(a.eps24u, p2);
    float fl = __fmaf_rn(a.e24lo, p2, __fmaf_rn(a.eps24u, p2l, __fmaf_rn(a.eps24u, p2, -fh)));
    // energy (measure pass only): from the two-float s6 in double precision
    double uu = 0.0;
    if (ENERGY) {
        const double s6d = (double)s6 + (double)s6l;
        uu = (double)a.eps4 * s6d * (s6d - 1.0);
    }
    if (COUL) {
        const float qi = __int_as_float(ri.w), qj = __int_as_float(rj.w);
        const float qh = __fmul_rn(qi, qj), ql = __fmaf_rn(qi, qj, -qh);
        const float kh = __fmul_rn(a.kcu, qh);
        const float kl = __fmaf_rn(a.kclo, qh, __fmaf_rn(a.kcu, ql, __fmaf_rn(a.kcu, qh, -kh)));
        // 1/r = ir + irl: the residual of ir^2 against ir2 and eta
        const float eir = __fmaf_rn(ir, ir, -ir2);
        const float irl = __fmul_rn(__fmul_rn(0.5f, ir), __fmaf_rn(-eir, r2, eta));
        const float i3 = __fmul_rn(ir, ir2);
        const float i3l = __fmaf_rn(irl, ir2, __fmaf_rn(ir, ir2l, __fmaf_rn(ir, ir2, -i3)));
        const float ch = __fmul_rn(kh, i3);
        const float cl2 = __fmaf_rn(kl, i3, __fmaf_rn(kh, i3l, __fmaf_rn(kh, i3, -ch)));
        const float sh = __fadd_rn(fh, ch);
        const float sb = __fsub_rn(sh, fh);
        const float se = __fadd_rn(__fsub_rn(fh, __fsub_rn(sh, sb)), __fsub_rn(ch, sb));
        fh = sh;
        fl = __fadd_rn(fl, __fadd_rn(cl2, se));
        if (ENERGY) uu += (double)a.kceu * ((double)qi * (double)qj) * ((double)ir + (double)irl);
    }
    // components fmag * d, into the two-float sums
    {
        const float tx = __fmul_rn(fh, dxh);
        df_acc(acc.xh, acc.xl, tx, __fmaf_rn(fl, dxh, __fmaf_rn(fh, dxl, __fmaf_rn(fh, dxh, -tx))));
        const float ty = __fmul_rn(fh, dyh);
        df_acc(acc.yh, acc.yl, ty, __fmaf_rn(fl, dyh, __fmaf_rn(fh, dyl, __fmaf_rn(fh, dyh, -ty))));
        const float tz = __fmul_rn(fh, dzh);
        df_acc(acc.zh, acc.zl, tz, __fmaf_rn(fl, dzh, __fmaf_rn(fh, dzl, __fmaf_rn(fh, dzh, -tz))));
    }
    if (ENERGY) ue += uu;
}

// Pair (i, j) from fixed-point records: the integer difference is exact, its
// conversion to float rounds once, so r_ij keeps full single precision at any
// box size inside the frame.  Constants are pre-scaled, so the force comes out
// in physical units per fixed-point unit of displacement.  Returns true,
// adding nothing, for a pair closer than 1.3 sigma (one that came near after
// the list build) or within a few ulps of the cutoff (where single precision
// cannot decide it): the caller evaluates it with accum_near.
template <bool COUL, bool ENERGY>
__device__ __forceinline__ bool accum_pair(const int4& ri, const int4& rj, const PairK& a,
                                          float& fx, float& fy, float& fz, double& ue) {
    const float dx = (float)idiff(ri.x, rj.x);
    const float dy = (float)idiff(ri.y, rj.y);
    const float dz = (float)idiff(ri.z, rj.z);
    const float r2 = dx * dx + dy * dy + dz * dz;
    if ((r2 < a.rn2u) | (fabsf(r2 - a.rc2u) <= a.band())) return true;
    if (r2 < a.rc2u) {
        float inv_r2, inv_r = 0.f;
        if (COUL) {
            inv_r = rsqrtf(r2);
            inv_r = inv_r * (1.5f - 0.5f * r2 * inv_r * inv_r);  // one Newton step
            inv_r2 = inv_r * inv_r;
        } else {
            inv_r2 = __fdividef(1.0f, r2);
            inv_r2 = inv_r2 * (2.0f - r2 * inv_r2);  // one Newton step
        }
        const float s2 = a.sig2u * inv_r2;
        const float s6 = s2 * s2 * s2;
        float fmag = a.eps24u * inv_r2 * s6 * (2.0f * s6 - 1.0f);
        if (COUL) {
            const float qq = __int_as_float(ri.w) * __int_as_float(rj.w);
            fmag += a.kcu * qq * inv_r * inv_r2;
        }
        fx += fmag * dx;
        fy += fmag * dy;
        fz += fmag * dz;
        if (ENERGY) {
            // the measure pass: the energy in double precision from the exact
            // integer separation (single-precision terms carry a systematic
            // bias of a fraction of an ulp, which ten million pairs add up)
            const double xd = (double)idiff(ri.x, rj.x), yd = (double)idiff(ri.y, rj.y),
                         zd = (double)idiff(ri.z, rj.z);
            // 1/r^2 and 1/r by two Newton-Raphson steps each in double
            // precision (y <- y (2 - r^2 y), y <- y (3 - r^2 y^2) / 2) from the
            // single-precision reciprocal and reciprocal square root: a double
            // division or square root costs several times more on GB300's FP64
            // pipe, and these terms run for every pair of the pass
            const double r2d = xd * xd + yd * yd + zd * zd;
            double ir2d = (double)__frcp_rn((float)r2d);
            ir2d = ir2d * (2.0 - r2d * ir2d);
            ir2d = ir2d * (2.0 - r2d * ir2d);
            const double s2d = ((double)a.sig2u + (double)a.sig2lo) * ir2d;
            const double s6d = s2d * s2d * s2d;
            double ud = (double)a.eps4 * s6d * (s6d - 1.0);
            if (COUL) {
                double ird = (double)rsqrtf((float)r2d);
                ird = ird * (1.5 - 0.5 * r2d * ird * ird);
                ird = ird * (1.5 - 0.5 * r2d * ird * ird);
                ud += (double)a.kceu * ((double)__int_as_float(ri.w) * (double)__int_as_float(rj.w)) *
                      ird;
            }
            ue += ud;
        }
    }
    return false;
}

// Pair constants of PairK, each in both halves.
struct PairK2 {
    uint64_t rc2u, sig2u, eps24u, kcu, two, mone, half_neg, three_half;
    __device__ __forceinline__ explicit PairK2(const PairK& a)
        : rc2u(pk2(a.rc2u, a.rc2u)), sig2u(pk2(a.sig2u, a.sig2u)),
          eps24u(pk2(a.eps24u, a.eps24u)), kcu(pk2(a.kcu, a.kcu)), two(pk2(2.0f, 2.0f)),
          mone(pk2(-1.0f, -1.0f)), half_neg(pk2(-0.5f, -0.5f)), three_half(pk2(1.5f, 1.5f)) {}
};


// (h, l) += the two halves of (H, L), a half at a time
__device__ __forceinline__ void df_fold2(float& h, float& l, uint64_t H, uint64_t L) {
    float ha, hb, la, lb;
    upk2(H, ha, hb);
    upk2(L, la, lb);
    df_acc(h, l, ha, la);
    df_acc(h, l, hb, lb);
}

// Separation parts of one near entry: hi (exact float of the masked coarse
// difference), lo (exact), fine (exact), per axis.
__device__ __forceinline__ void near_parts(const int4& ri, const int4& rj, const uint2& fi,
                                           const uint2& fj, int32_t hmask, float h[3], float l[3],
                                           float f[3]) {
    const int32_t ix = idiff(ri.x, rj.x), iy = idiff(ri.y, rj.y), iz = idiff(ri.z, rj.z);
    h[0] = __int2float_rn(ix & hmask); l[0] = lo_part(ix & ~hmask);
    h[1] = __int2float_rn(iy & hmask); l[1] = lo_part(iy & ~hmask);
    h[2] = __int2float_rn(iz & hmask); l[2] = lo_part(iz & ~hmask);
    f[0] = fine_diff(fi.x, fj.x, 0);
    f[1] = fine_diff(fi.x, fj.x, 16);
    f[2] = fine_diff(fi.y, fj.y, 0);
}

// accum_near for two near entries (i, a) and (i, b) at once (no energies):
// the same operations in the same order on both halves of packed registers
// (add/sub/mul/fma.rn.f32x2 round each half as the scalar form does), so each
// entry's term has the scalar form's bits; the two terms are then added to
// the two-float sums one after the other, as the scalar form adds them.
template <bool COUL>
__device__ __forceinline__ void accum_near2(const int4& ri, const int4& ra, const int4& rb,
                                            const uint2& fi, const uint2& fa, const uint2& fb,
                                            const PairK& a, DF3& acc) {
    float ha[3], la[3], fa3[3], hb[3], lb[3], fb3[3];
    near_parts(ri, ra, fi, fa, a.hmask, ha, la, fa3);
    near_parts(ri, rb, fi, fb, a.hmask, hb, lb, fb3);
    uint64_t H[3], Lo[3], F[3], DH[3], DL[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        H[d] = pk2(ha[d], hb[d]);
        Lo[d] = pk2(la[d], lb[d]);
        F[d] = pk2(fa3[d], fb3[d]);
        DH[d] = add2(H[d], Lo[d]);
        DL[d] = add2(sub2(Lo[d], sub2(DH[d], H[d])), F[d]);
    }
    const uint64_t two = sp2(2.0f), one = sp2(1.0f);
    const uint64_t P = fma2(H[2], H[2], fma2(H[1], H[1], mul2(H[0], H[0])));  // exact
    const uint64_t t = fma2(H[0], Lo[0], fma2(H[1], Lo[1], mul2(H[2], Lo[2])));
    const uint64_t l2 = fma2(Lo[0], Lo[0], fma2(Lo[1], Lo[1], mul2(Lo[2], Lo[2])));
    const uint64_t u = fma2(DH[0], F[0], fma2(DH[1], F[1], mul2(DH[2], F[2])));
    const uint64_t cl = fma2(two, u, fma2(two, t, l2));
    const uint64_t r2 = add2(P, cl);
    const uint64_t r2lo = sub2(cl, sub2(r2, P));
    float da, db;
    upk2(add2(sub2(r2, sp2(a.rc2u)), sub2(r2lo, sp2(a.rc2lo))), da, db);
    const bool ina = da < 0.0f, inb = db < 0.0f;
    if (!(ina | inb)) return;
    float r2a, r2b;
    upk2(r2, r2a, r2b);
    const uint64_t ir = pk2(rsqrtf(r2a), rsqrtf(r2b));
    const uint64_t ir2 = mul2(ir, ir);
    const uint64_t eta = fma2(neg2(r2lo), ir2, fma2(neg2(r2), ir2, one));
    const uint64_t ir2l = mul2(ir2, eta);
    const uint64_t sg = sp2(a.sig2u);
    const uint64_t s2 = mul2(sg, ir2);
    const uint64_t s2l = fma2(sp2(a.sig2lo), ir2, fma2(sg, ir2l, fma2(sg, ir2, neg2(s2))));
    const uint64_t s4 = mul2(s2, s2);
    const uint64_t s4l = fma2(mul2(two, s2), s2l, fma2(s2, s2, neg2(s4)));
    const uint64_t s6 = mul2(s4, s2);
    const uint64_t s6l = fma2(s4, s2l, fma2(s4l, s2, fma2(s4, s2, neg2(s6))));
    const uint64_t a2 = mul2(two, s6);
    const uint64_t wh = sub2(a2, one);
    const uint64_t wb = sub2(wh, a2);
    const uint64_t we = add2(sub2(a2, sub2(wh, wb)), sub2(neg2(one), wb));
    const uint64_t wl = fma2(two, s6l, we);
    const uint64_t p1 = mul2(ir2, s6);
    const uint64_t p1l = fma2(ir2l, s6, fma2(ir2, s6l, fma2(ir2, s6, neg2(p1))));
    const uint64_t p2 = mul2(p1, wh);
    const uint64_t p2l = fma2(p1l, wh, fma2(p1, wl, fma2(p1, wh, neg2(p2))));
    const uint64_t e24 = sp2(a.eps24u);
    uint64_t fh = mul2(e24, p2);
    uint64_t fl = fma2(sp2(a.e24lo), p2, fma2(e24, p2l, fma2(e24, p2, neg2(fh))));
    if (COUL) {
        const float qi = __int_as_float(ri.w), qa = __int_as_float(ra.w), qb = __int_as_float(rb.w);
        const float qha = __fmul_rn(qi, qa), qhb = __fmul_rn(qi, qb);
        const uint64_t qh = pk2(qha, qhb);
        const uint64_t ql = pk2(__fmaf_rn(qi, qa, -qha), __fmaf_rn(qi, qb, -qhb));
        const uint64_t kc = sp2(a.kcu);
        const uint64_t kh = mul2(kc, qh);
        const uint64_t kl = fma2(sp2(a.kclo), qh, fma2(kc, ql, fma2(kc, qh, neg2(kh))));
        const uint64_t eir = fma2(ir, ir, neg2(ir2));
        const uint64_t irl = mul2(mul2(sp2(0.5f), ir), fma2(neg2(eir), r2, eta));
        const uint64_t i3 = mul2(ir, ir2);
        const uint64_t i3l = fma2(irl, ir2, fma2(ir, ir2l, fma2(ir, ir2, neg2(i3))));
        const uint64_t ch = mul2(kh, i3);
        const uint64_t cl2 = fma2(kl, i3, fma2(kh, i3l, fma2(kh, i3, neg2(ch))));
        const uint64_t sh = add2(fh, ch);
        const uint64_t sb = sub2(sh, fh);
        const uint64_t se = add2(sub2(fh, sub2(sh, sb)), sub2(ch, sb));
        fh = sh;
        fl = add2(fl, add2(cl2, se));
    }
    if (!(ina & inb)) {
        // one entry beyond the cutoff: its half contributes zero
        float x0, x1, y0, y1;
        upk2(fh, x0, x1);
        upk2(fl, y0, y1);
        fh = pk2(ina ? x0 : 0.0f, inb ? x1 : 0.0f);
        fl = pk2(ina ? y0 : 0.0f, inb ? y1 : 0.0f);
    }
    const uint64_t tx = mul2(fh, DH[0]);
    df_fold2(acc.xh, acc.xl, tx, fma2(fl, DH[0], fma2(fh, DL[0], fma2(fh, DH[0], neg2(tx)))));
    const uint64_t ty = mul2(fh, DH[1]);
    df_fold2(acc.yh, acc.yl, ty, fma2(fl, DH[1], fma2(fh, DL[1], fma2(fh, DH[1], neg2(ty)))));
    const uint64_t tz = mul2(fh, DH[2]);
    df_fold2(acc.zh, acc.zl, tz, fma2(fl, DH[2], fma2(fh, DL[2], fma2(fh, DH[2], neg2(tz)))));
}

// Forces of the pairs (i, a) and (i, b) together (no energies): the same
// terms as accum_pair, the pair outside the cutoff contributing zero.  The
// accumulators hold the running sums of the a-entries and the b-entries
// separately; the caller adds the halves at the end.  When a pair is closer
// than 1.3 sigma (rare: one that came near after the list build) or lies
// within a few ulps of the cutoff, the other takes the scalar form into (sx,
// sy, sz) and that one is left to the caller: the return value has bit 0 set
// for a, bit 1 for b.
template <bool COUL>
__device__ __forceinline__ unsigned accum_pair2(const int4& ri, const int4& ra, const int4& rb,
                                               const PairK& k1, const PairK2& k, uint64_t& fx,
                                               uint64_t& fy, uint64_t& fz, float& sx, float& sy,
                                               float& sz) {
    const uint64_t dx = pk2((float)idiff(ri.x, ra.x), (float)idiff(ri.x, rb.x));
    const uint64_t dy = pk2((float)idiff(ri.y, ra.y), (float)idiff(ri.y, rb.y));
    const uint64_t dz = pk2((float)idiff(ri.z, ra.z), (float)idiff(ri.z, rb.z));
    const uint64_t r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
    float r2a, r2b;
    upk2(r2, r2a, r2b);
    const float band = k1.band();
    if ((r2a < k1.rn2u) | (r2b < k1.rn2u) | (fabsf(r2a - k1.rc2u) <= band) |
        (fabsf(r2b - k1.rc2u) <= band)) {
        double ue = 0.0;
        unsigned m = accum_pair<COUL, false>(ri, ra, k1, sx, sy, sz, ue) ? 1u : 0u;
        m |= accum_pair<COUL, false>(ri, rb, k1, sx, sy, sz, ue) ? 2u : 0u;
        return m;
    }
    // no early return when both lie beyond the cutoff: the zeroed terms cost
    // less than the divergent branch
    const bool ina = r2a < k1.rc2u, inb = r2b < k1.rc2u;
    uint64_t inv_r = 0, inv_r2;
    if (COUL) {
        inv_r = pk2(rsqrtf(r2a), rsqrtf(r2b));
        // one Newton step: inv_r (1.5 - 0.5 r2 inv_r^2)
        const uint64_t t = fma2(k.half_neg, mul2(r2, mul2(inv_r, inv_r)), k.three_half);
        inv_r = mul2(inv_r, t);
        inv_r2 = mul2(inv_r, inv_r);
    } else {
        inv_r2 = pk2(__fdividef(1.0f, r2a), __fdividef(1.0f, r2b));
        // one Newton step: inv_r2 (2 - r2 inv_r2)
        inv_r2 = mul2(inv_r2, fma2(mul2(r2, inv_r2), k.mone, k.two));
    }
    const uint64_t s2 = mul2(k.sig2u, inv_r2);
    const uint64_t s6 = mul2(mul2(s2, s2), s2);
    uint64_t fmag = mul2(mul2(mul2(k.eps24u, inv_r2), s6), fma2(k.two, s6, k.mone));
    if (COUL) {
        const float qi = __int_as_float(ri.w);
        const uint64_t qq = pk2(qi * __int_as_float(ra.w), qi * __int_as_float(rb.w));
        fmag = fma2(mul2(k.kcu, qq), mul2(inv_r, inv_r2), fmag);
    }
    float fa, fb;
    upk2(fmag, fa, fb);
    fmag = pk2(ina ? fa : 0.0f, inb ? fb : 0.0f);
    fx = fma2(fmag, dx, fx);
    fy = fma2(fmag, dy, fy);
    fz = fma2(fmag, dz, fz);
    return 0u;
}

// One block per 256 atoms.  MODE 0: step (force, pending half kick, kick,
// drift, reflect, next record).  MODE 2: the same step inside a captured
// window, whose last block also sets the early-refit condition of the graph
// node after it.  MODE 1: measure (force, integer-step velocity and
// energies; state untouched).  MODE 3: measure without the potential energy
// (forces and velocities for a read-back or a thermostat: the double-precision
// pair energies are most of a measure pass's time).
// BATCH: atoms of several systems; pair constants, walls and the fixed-point
// origin come from the atom's system (a pair never crosses systems).
// TPA: threads per atom.  With TPA > 1 (small systems, whose grid is under a
// couple of waves) thread p of an atom sums list entries p, p + TPA, ... and
// the slices are added in a fixed order before the atom's update.
template <bool COUL, int MODE, bool BATCH, int TPA = 1, int SPLIT = 1>
__global__ void __launch_bounds__(kBlock * TPA / SPLIT, TPA == 1 ? 4 : 1) k_md_step(StepArgs a) {
    extern __shared__ int4 srec[];
    // MODE 1 and 3 measure (3: without the potential energy)
    constexpr bool MEASURE = MODE == 1 || MODE == 3;
    // SPLIT thread blocks share a block of kBlock atoms (and its lists), each
    // taking kBlock / SPLIT of them
    constexpr int APB = kBlock / SPLIT;
    const int32_t blk = (int32_t)(blockIdx.x / SPLIT);
    const int tid = (int)(blockIdx.x % SPLIT) * APB + (int)(threadIdx.x & (APB - 1));  // the atom
    const int part = threadIdx.x / APB;  // its list slice
    int64_t i = (int64_t)blk * kBlock + tid;
    const bool valid = i < a.n;
    const bool own = part == 0;  // the thread that updates the atom
    const int32_t* __restrict__ U = a.ulist + (int64_t)blk * a.ucap;
    // stage the block's union: record of atom (leaf * apl + e) at u * apl + e,
    // up to the shared-memory capacity; larger unions read the rest from L2
    {
        // four records per thread in flight: their leaf indices, then the
        // records (apl is a power of two)
        const int32_t nu = min(__ldg(&a.ucount[blk]), a.ucap);
        const int32_t m = min(nu * a.apl, a.smrec);
        const int32_t lsh = __ffs(a.apl) - 1, emask = a.apl - 1;
        constexpr int32_t NT = APB * TPA;
        for (int32_t k = threadIdx.x; k < m; k += 4 * NT) {
            int32_t lf[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int32_t kk = k + j * NT;
                lf[j] = kk < m ? __ldg(&U[kk >> lsh]) : 0;
            }
            int4 r[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int32_t kk = k + j * NT;
                if (kk < m) r[j] = __ldg(&a.rec_in[((int64_t)lf[j] << lsh) + (kk & emask)]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int32_t kk = k + j * NT;
                if (kk < m) srec[kk] = r[j];
            }
        }
    }
    __syncthreads();
    // idle lanes (last block) run with an empty list and store nothing; they
    // join the warp reductions (measure) and the block vote (step)
    if (!valid) i = a.n - 1;
    const int4 ri = __ldg(&a.rec_in[i]);
    PairK pk{a.rc2u, a.sig2u, a.eps24u, a.eps4, a.kcu, a.kceu,
             a.nk.rn2u, a.nk.sig2lo, a.nk.e24lo, a.nk.kclo, a.nk.rc2lo, a.nk.hmask};
    int32_t sv = 0;
    const SysRow* __restrict__ row = nullptr;
    double S = a.fr.s;
    float hs2u = a.half_skin2u, hsu = a.hsu;
    if constexpr (BATCH) {
        sv = __ldg(&a.sid[i]);
        row = a.sys + sv;
        pk.sig2u = __ldg(&row->sig2u);
        pk.eps24u = __ldg(&row->eps24u);
        pk.eps4 = __ldg(&row->eps4);
        pk.rc2u = __ldg(&row->rc2u);
        pk.kcu = __ldg(&row->kcu);
        pk.kceu = __ldg(&row->kceu);
        pk.rn2u = __ldg(&row->nk.rn2u);
        pk.sig2lo = __ldg(&row->nk.sig2lo);
        pk.e24lo = __ldg(&row->nk.e24lo);
        pk.kclo = __ldg(&row->nk.kclo);
        pk.rc2lo = __ldg(&row->nk.rc2lo);
        pk.hmask = __ldg(&row->nk.hmask);
        S = __ldg(&row->s);
        hs2u = __ldg(&row->hs2u);
        hsu = __ldg(&row->hsu);
    }
    // near entries (slots 0, 1, ...) and the others (slots lcap - 1, lcap - 2, ...)
    const int32_t cpk = valid ? __ldg(&a.ncount[i]) : 0;
    const int32_t nn = list_near(cpk), nf = cpk >> 16;
    const uint16_t* __restrict__ L = a.llist + (int64_t)blk * a.lcap * kBlock + tid;
    const uint16_t* __restrict__ LF = L + (int64_t)(a.lcap - 1) * kBlock;
    const int32_t lsh = __ffs(a.apl) - 1, emask = a.apl - 1;
    const uint2 fi = __ldg(&a.recf_in[i]);
    // near terms in two-float sums, the others in single precision
    DF3 nacc{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float fx = 0.f, fy = 0.f, fz = 0.f;
    double ue = 0.0;  // potential energy (measure pass only)
    __shared__ float spart[TPA > 1 ? TPA - 1 : 1][8][kBlock];
    // The pair loops, compiled twice: for a block whose whole union is staged
    // (the usual case; a block-uniform choice) a record is read from shared
    // memory with no test, otherwise records past the staged part come from L2.
    auto pairs = [&](auto staged) {
        constexpr bool ALL = decltype(staged)::value;
        auto fetch = [&](int32_t li) -> int4 {
            if (ALL || li < a.smrec) return srec[li];
            return __ldg(&a.rec_in[((int64_t)__ldg(&U[li >> lsh]) << lsh) + (li & emask)]);
        };
        // fine bits of a union entry's record (near pairs only)
        auto fine = [&](int32_t li) -> uint2 {
            return __ldg(&a.recf_in[((int64_t)__ldg(&U[li >> lsh]) << lsh) + (li & emask)]);
        };
        if constexpr (MEASURE || BATCH) {
            // near entries of this thread's slice, the next index loaded ahead
            // (the measure pass, and ensembles, whose per-system constants leave
            // no registers for the packed form)
            int32_t s = part;
            int32_t li = s < nn ? L[(int64_t)s * kBlock] : 0;
            for (; s < nn; s += TPA) {
                const int32_t sn = s + TPA;
                const int32_t next = sn < nn ? L[(int64_t)sn * kBlock] : 0;
                accum_near<COUL, MODE == 1>(ri, fetch(li), fi, fine(li), pk, nacc, ue);
                li = next;
            }
        } else {
            // near entries of this thread's slice two at a time (packed), the
            // next two indices loaded ahead; an odd last one alone
            int32_t s = part;
            int32_t la = s < nn ? L[(int64_t)s * kBlock] : 0;
            int32_t lb = s + TPA < nn ? L[(int64_t)(s + TPA) * kBlock] : 0;
            for (; s + TPA < nn; s += 2 * TPA) {
                const int32_t s2 = s + 2 * TPA;
                const int4 ra = fetch(la), rb = fetch(lb);
                const uint2 fa = fine(la), fb = fine(lb);
                la = s2 < nn ? L[(int64_t)s2 * kBlock] : 0;
                lb = s2 + TPA < nn ? L[(int64_t)(s2 + TPA) * kBlock] : 0;
                accum_near2<COUL>(ri, ra, rb, fi, fa, fb, pk, nacc);
            }
            if (s < nn) accum_near<COUL, false>(ri, fetch(la), fi, fine(la), pk, nacc, ue);
        }
        // an entry of the other segment that came closer than 1.3 sigma
        auto far_near = [&](int32_t s) {
            const int32_t li = LF[-(int64_t)s * kBlock];
            accum_near<COUL, MODE == 1>(ri, fetch(li), fi, fine(li), pk, nacc, ue);
        };
        if constexpr (TPA == 1) {
            // groups of four neighbours; the next group's indices are loaded
            // while the current group is computed
            const PairK2 pk2c(pk);
            [[maybe_unused]] uint64_t fx2 = 0, fy2 = 0, fz2 = 0;  // packed (0.0f, 0.0f)
            [[maybe_unused]] float gx = 0.f, gy = 0.f, gz = 0.f;  // measure pass: odd entries
            int32_t s = 0;
            int32_t li[4];
            if (nf >= 4) {
#pragma unroll
                for (int k = 0; k < 4; ++k) li[k] = LF[-(int64_t)k * kBlock];
            }
            for (; s + 4 <= nf; s += 4) {
                int4 rj[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) rj[k] = fetch(li[k]);
                if (s + 8 <= nf) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) li[k] = LF[-(int64_t)(s + 4 + k) * kBlock];
                }
                if constexpr (MEASURE) {
                    // even entries into (fx, fy, fz), odd ones into (gx, gy, gz),
                    // as the two halves of the packed form
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const bool nr = (k & 1) ? accum_pair<COUL, MODE == 1>(ri, rj[k], pk, gx, gy, gz, ue)
                                                : accum_pair<COUL, MODE == 1>(ri, rj[k], pk, fx, fy, fz, ue);
                        if (nr) far_near(s + k);
                    }
                } else {
                    // two entries per packed instruction
                    const unsigned m0 = accum_pair2<COUL>(ri, rj[0], rj[1], pk, pk2c, fx2, fy2,
                                                          fz2, fx, fy, fz);
                    const unsigned m1 = accum_pair2<COUL>(ri, rj[2], rj[3], pk, pk2c, fx2, fy2,
                                                          fz2, fx, fy, fz);
                    if (m0 | m1) {
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (((k < 2 ? m0 : m1) >> (k & 1)) & 1u) far_near(s + k);
                    }
                }
            }
            if constexpr (!MEASURE) {
                float a, b;
                upk2(fx2, a, b); fx += a + b;
                upk2(fy2, a, b); fy += a + b;
                upk2(fz2, a, b); fz += a + b;
            } else {
                fx += gx;
                fy += gy;
                fz += gz;
            }
            for (; s < nf; ++s)
                if (accum_pair<COUL, MODE == 1>(ri, fetch(LF[-(int64_t)s * kBlock]), pk, fx, fy,
                                                fz, ue))
                    far_near(s);
            // the force: two-float near sums with the single-precision sums added
            // to their low parts, rounded once
            fx = __fadd_rn(nacc.xh, __fadd_rn(nacc.xl, fx));
            fy = __fadd_rn(nacc.yh, __fadd_rn(nacc.yl, fy));
            fz = __fadd_rn(nacc.zh, __fadd_rn(nacc.zl, fz));
        } else {
            // slice `part` of the far entries (part, part + TPA, ..., in that
            // order): four indices loaded ahead while the previous four are computed
            int32_t li[4] = {0, 0, 0, 0};
            auto load4 = [&](int32_t s0) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int32_t sk = s0 + k * TPA;
                    li[k] = sk < nf ? LF[-(int64_t)sk * kBlock] : 0;
                }
            };
            int32_t s = part;
            if (s < nf) load4(s);
            for (; s + 3 * TPA < nf; s += 4 * TPA) {
                int4 rj[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) rj[k] = fetch(li[k]);
                load4(s + 4 * TPA);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (accum_pair<COUL, MODE == 1>(ri, rj[k], pk, fx, fy, fz, ue))
                        far_near(s + k * TPA);
            }
            // at most three entries left, their indices already loaded
            for (int k = 0; s < nf && k < 4; s += TPA, ++k)
                if (accum_pair<COUL, MODE == 1>(ri, fetch(li[k]), pk, fx, fy, fz, ue)) far_near(s);
            // each slice as a two-float value (its single-precision sum in the low
            // part); the slices added in a fixed order
            nacc.xl = __fadd_rn(nacc.xl, fx);
            nacc.yl = __fadd_rn(nacc.yl, fy);
            nacc.zl = __fadd_rn(nacc.zl, fz);
            if (part > 0) {
                spart[part - 1][0][tid] = nacc.xh;
                spart[part - 1][1][tid] = nacc.xl;
                spart[part - 1][2][tid] = nacc.yh;
                spart[part - 1][3][tid] = nacc.yl;
                spart[part - 1][4][tid] = nacc.zh;
                spart[part - 1][5][tid] = nacc.zl;
                const float uh = (float)ue;
                spart[part - 1][6][tid] = uh;
                spart[part - 1][7][tid] = (float)(ue - (double)uh);
            }
            __syncthreads();
            if (own) {
#pragma unroll
                for (int p = 0; p < TPA - 1; ++p) {
                    df_acc(nacc.xh, nacc.xl, spart[p][0][tid], spart[p][1][tid]);
                    df_acc(nacc.yh, nacc.yl, spart[p][2][tid], spart[p][3][tid]);
                    df_acc(nacc.zh, nacc.zl, spart[p][4][tid], spart[p][5][tid]);
                    ue += (double)spart[p][6][tid] + (double)spart[p][7][tid];
                }
            }
            fx = __fadd_rn(nacc.xh, nacc.xl);
            fy = __fadd_rn(nacc.yh, nacc.yl);
            fz = __fadd_rn(nacc.zh, nacc.zl);
        }
    };
    if (min(__ldg(&a.ucount[blk]), a.ucap) * a.apl <= a.smrec)
        pairs(std::true_type{});
    else
        pairs(std::false_type{});
    if (valid && own) a.f_out[i] = make_float4(fx, fy, fz, 0.f);
    const bool MASS = a.has_mass != 0, FIRST = a.first != 0;
    const double imv = MASS ? a.im[i] : 1.0;
    const float fv[3] = {fx, fy, fz};
    if constexpr (MEASURE) {
        double ke = 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double kick = (double)(a.hdt * fv[d]) * imv;
            double v = FIRST ? a.w[d][i] : a.w[d][i] + kick;
            if (valid && own) a.v_out[d][i] = v;
            ke += v * v;
        }
        double mass = MASS ? 1.0 / imv : 1.0;
        double pe = valid && own ? 0.5 * (double)ue : 0.0;
        ke = valid && own ? ke * 0.5 * mass : 0.0;
        // per-system sums (one system unless batched); a warp spanning two
        // systems adds lane by lane
        if (BATCH && !__all_sync(0xffffffffu, sv == __shfl_sync(0xffffffffu, sv, 0))) {
            if (valid) {
                atomicAdd(&a.acc[2 * sv], pe);
                atomicAdd(&a.acc[2 * sv + 1], ke);
            }
            return;
        }
        for (int sh = 16; sh > 0; sh >>= 1) {
            pe += __shfl_xor_sync(0xffffffffu, pe, sh);
            ke += __shfl_xor_sync(0xffffffffu, ke, sh);
        }
        if ((tid & 31) == 0) {
            atomicAdd(&a.acc[2 * sv], pe);
            atomicAdd(&a.acc[2 * sv + 1], ke);
        }
        return;
    } else {
        // v_{n+1/2} = v_{n-1/2} + dt F/m (the pending half kick and this step's
        // half kick in one add), x += dt v, walls, next record.
        const float kdt = FIRST ? a.hdt : 2.0f * a.hdt;
        int32_t xi[3];
        uint32_t xf[3];
        bool trig = false;
        if (valid && own) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double v = a.w[d][i] + (double)(kdt * fv[d]) * imv;
            double x = fma(a.dt, v, a.x[d][i]);
            const double os = BATCH ? __ldg(&row->os[d]) : a.os[d];
            long long q = __double2ll_rn(fma(x, S * kFine, -os));
            // integer pre-check (before the wrap); the exact FP64 test of
            // boundary_reflect! runs only for atoms within a grid step of a wall
            const int64_t lfp = BATCH ? __ldg(&row->lo_fp[d]) : a.lo_fp[d];
            const int64_t hfp = BATCH ? __ldg(&row->hi_fp[d]) : a.hi_fp[d];
            if (q <= lfp + 1 || q >= hfp - 1) {
                const double lo = BATCH ? __ldg(&row->lo[d]) : a.lo[d];
                const double hi = BATCH ? __ldg(&row->hi[d]) : a.hi[d];
                if (lo > x) { v = -v; x = lo; }
                if (hi < x) { v = -v; x = hi; }
                q = __double2ll_rn(fma(x, S * kFine, -os));
                if (!(x == x)) set_error(a.err, ND_ERR_NONFINITE, (int32_t)i);
            }
            a.x[d][i] = x;
            a.w[d][i] = v;
            xi[d] = (int32_t)(uint32_t)(unsigned long long)(q >> 16);
            xf[d] = (uint32_t)q & 0xffffu;
        }
        a.rec_out[i] = make_int4(xi[0], xi[1], xi[2], ri.w);
        a.recf_out[i] = pack_fine(xf[0], xf[1], xf[2]);
        // A list built at r_c + skin stays valid while no atom moved more than
        // skin/2 since the build; count the atom-steps that broke that bound
        // where the next step keeps the list without a check.
        const int4 rb = __ldg(&a.rec_build[i]);
        const float ex = (float)idiff(xi[0], rb.x), ey = (float)idiff(xi[1], rb.y),
                    ez = (float)idiff(xi[2], rb.z);
        const float e2 = ex * ex + ey * ey + ez * ez;
        if (a.unchecked && e2 > hs2u) atomicAdd(a.diag, 1ull);
        // Ask for a refit before the next step when this atom could pass the
        // bound before the next check: displacement so far + trig_k times this
        // step's move + 5% of the bound (no step until the next check moves
        // it more than twice as far as this one; with a check after every
        // step, trig_k = 2 still covers one step more).
        if (a.vote) {
            const float sx = (float)idiff(xi[0], ri.x), sy = (float)idiff(xi[1], ri.y),
                        sz = (float)idiff(xi[2], ri.z);
            trig = sqrtf(e2) + a.trig_k * sqrtf(sx * sx + sy * sy + sz * sz) > 0.95f * hsu;
        }
        }
        // Early refit request: the block votes, and the last block to finish
        // (a ticket counter, no waiting) publishes the flag to the graph's
        // conditional node that follows this step.
        if (__syncthreads_or(trig) && threadIdx.x == 0) atomicOr(&a.ctl[0], 1u);
        if constexpr (MODE == 2) {
            if (threadIdx.x == 0) {
                __threadfence();
                const unsigned ticket = atomicAdd(&a.ctl[1], 1u);
                if (ticket == gridDim.x - 1) {
                    __threadfence();
                    const unsigned f = atomicExch(&a.ctl[0], 0u);
                    atomicExch(&a.ctl[1], 0u);
                    cudaGraphSetConditional(a.cond, f ? 1u : 0u);
                }
            }
        }
    }
}

__global__ void k_md_unsort(const int32_t* __restrict__ orig, int32_t n, const double* x0,
                            const double* x1, const double* x2, const double* v0,
                            const double* v1, const double* v2, const float4* __restrict__ f,
                            double* xo, double* vo, float* fo) {
    int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int64_t o = orig[k];
    if (xo) { xo[3 * o] = x0[k]; xo[3 * o + 1] = x1[k]; xo[3 * o + 2] = x2[k]; }
    if (vo) { vo[3 * o] = v0[k]; vo[3 * o + 1] = v1[k]; vo[3 * o + 2] = v2[k]; }
    if (fo) { float4 g = f[k]; fo[3 * o] = g.x; fo[3 * o + 1] = g.y; fo[3 * o + 2] = g.z; }
}

// Reference call shape: forces over an explicit (1-based) pair list, physical
// units; displacement from hi/lo float splits of the FP64 positions.
__device__ __forceinline__ void split_df(double x, float& hi, float& lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}

__global__ void k_pair_forces(const double* __restrict__ x, const double* __restrict__ q,
                              const int32_t* __restrict__ pi, const int32_t* __restrict__ pj,
                              int64_t np, int32_t n, float rc2, float sig2, float eps24,
                              float eps4, float kc, float* __restrict__ f, double* acc,
                              int32_t* err) {
    double ue = 0.0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < np;
         k += (int64_t)gridDim.x * blockDim.x) {
        int32_t i = pi[k] - 1, j = pj[k] - 1;
        if (i < 0 || j < 0 || i >= n || j >= n) { set_error(err, ND_ERR_ARG, (int32_t)k); continue; }
        float h[6], l[6];
        for (int d = 0; d < 3; ++d) {
            split_df(x[3 * (int64_t)i + d], h[d], l[d]);
            split_df(x[3 * (int64_t)j + d], h[3 + d], l[3 + d]);
        }
        float dx = (h[0] - h[3]) + (l[0] - l[3]);
        float dy = (h[1] - h[4]) + (l[1] - l[4]);
        float dz = (h[2] - h[5]) + (l[2] - l[5]);
        float r2 = dx * dx + dy * dy + dz * dz;
        if (!(r2 < rc2)) continue;
        float inv_r2 = 1.0f / r2;
        float s2 = sig2 * inv_r2;
        float s6 = s2 * s2 * s2;
        float fmag = eps24 * inv_r2 * s6 * (2.0f * s6 - 1.0f);
        float u = eps4 * s6 * (s6 - 1.0f);
        if (q) {
            float inv_r = rsqrtf(r2);
            inv_r = inv_r * (1.5f - 0.5f * r2 * inv_r * inv_r);
            float e = kc * (float)q[i] * (float)q[j] * inv_r;
            fmag += e * inv_r2;
            u += e;
        }
        ue += (double)u;
        atomicAdd(&f[3 * (int64_t)i], fmag * dx); atomicAdd(&f[3 * (int64_t)i + 1], fmag * dy);
        atomicAdd(&f[3 * (int64_t)i + 2], fmag * dz);
        atomicAdd(&f[3 * (int64_t)j], -fmag * dx); atomicAdd(&f[3 * (int64_t)j + 1], -fmag * dy);
        atomicAdd(&f[3 * (int64_t)j + 2], -fmag * dz);
    }
    for (int s = 16; s > 0; s >>= 1) ue += __shfl_xor_sync(0xffffffffu, ue, s);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, ue);
}

// ------------------------------------------------------------- engine


static nd_status md_alloc(MDEngine* m) {
    Ctx* c = &m->sub;
    const size_t n = (size_t)m->n;
    nd_status st;
    for (int s = 0; s < 2; ++s) {
        // x[3], w[3], q, im (8 doubles) + orig (int32) [+ sid (int32)]
        if ((st = ensure(c, m->set_buf[s], n * (8 * sizeof(double) + 2 * sizeof(int32_t)) + 256))) return st;
        double* b = (double*)m->set_buf[s].p;
        for (int d = 0; d < 3; ++d) { m->set[s].x[d] = b + d * n; m->set[s].w[d] = b + (3 + d) * n; }
        m->set[s].q = b + 6 * n;
        m->set[s].im = b + 7 * n;
        m->set[s].orig = (int32_t*)(b + 8 * n);
        m->set[s].sid = m->nsys > 0 ? m->set[s].orig + n : nullptr;
        if ((st = ensure(c, m->rec_buf[s], n * sizeof(int4)))) return st;
        if ((st = ensure(c, m->recf_buf[s], n * sizeof(uint2)))) return st;
    }
    if ((st = ensure(c, m->recb, n * sizeof(int4)))) return st;
    if ((st = ensure(c, m->lcount_leaf, sizeof(int32_t) * (size_t)m->nL))) return st;
    if ((st = ensure(c, m->xyz32, 3 * n * sizeof(float)))) return st;
    if ((st = ensure(c, m->pos32, n * sizeof(float4)))) return st;
    if ((st = ensure(c, m->keys, 32 * (size_t)(2 * m->nL)))) return st;
    if ((st = ensure(c, m->store, sizeof(int32_t) * (size_t)m->nL))) return st;
    if ((st = ensure(c, m->bbox, 32 * ((size_t)m->nblocks + (size_t)cdiv(m->nblocks, 32)))))
        return st;
    if ((st = ensure(c, m->ucount, sizeof(int32_t) * (size_t)m->nblocks))) return st;
    if ((st = ensure(c, m->ncount, sizeof(int32_t) * n))) return st;
    if ((st = ensure(c, m->f, sizeof(float4) * n))) return st;
    if ((st = ensure(c, m->vtmp, 3 * sizeof(double) * n))) return st;
    if ((st = ensure(c, m->acc, std::max<size_t>(64, 2 * sizeof(double) * (size_t)m->nsys)))) return st;
    if ((st = ensure(c, m->diag, 64))) return st;
    if (cudaMemsetAsync(m->diag.p, 0, 64, c->stream) != cudaSuccess) return ND_ERR_CUDA;
    if ((st = ensure(c, m->ctl, 64))) return st;
    if (cudaMemsetAsync(m->ctl.p, 0, 64, c->stream) != cudaSuccess) return ND_ERR_CUDA;
    if ((st = ensure(c, m->obs, 64))) return st;
    if (cudaMemsetAsync(m->obs.p, 0, 64, c->stream) != cudaSuccess) return ND_ERR_CUDA;
    if ((st = ensure(c, m->obs_part, sizeof(double) * (size_t)cdiv(m->n, 256)))) return st;
    // rebuild pipeline scratch: codes + perm + sort ping-pong + histograms
    if ((st = ensure(c, c->codes, sizeof(int32_t) * n))) return st;
    if ((st = ensure(c, c->perm, sizeof(int32_t) * n))) return st;
    if ((st = ensure(c, c->codes_alt, sizeof(uint32_t) * n))) return st;
    if ((st = ensure(c, c->perm_alt, sizeof(int32_t) * n))) return st;
    if ((st = ensure(c, c->hist, sizeof(uint32_t) * (256 * (size_t)cdiv(m->n, 2048) + 256)))) return st;
    if ((st = ensure(c, c->misc, 64))) return st;
    return ND_OK;
}

static cudaError_t raise_smem_limit(const void* fn, int maxsm) {
    cudaFuncAttributes fa{};
    cudaError_t e = cudaFuncGetAttributes(&fa, fn);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                maxsm - (int)fa.sharedSizeBytes);
}

// Union and list buffers for capacities (ucap, lcap), and the shared-memory
// opt-ins of the kernels that stage them.
static nd_status md_alloc_lists(MDEngine* m, int32_t fcap, int32_t ucap, int32_t lcap_leaf,
                                int32_t lcap, int32_t ucap_sm) {
    Ctx* c = &m->sub;
    nd_status st;
    m->fcap = fcap;
    m->ucap = ucap;
    m->lcap = lcap;
    m->lcap_leaf = lcap_leaf;
    m->ucap_sm = std::min(ucap_sm, ucap);
    int32_t p2 = 1;
    while (p2 < ucap) p2 <<= 1;
    m->upow2 = p2;
    int maxsm = 0;
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
    // staged records must fit the block's shared memory
    m->ucap_sm = std::max(0, std::min(m->ucap_sm, (maxsm - 1024) / (16 * m->apl)));
    if ((st = ensure(c, m->ulist, sizeof(int32_t) * (size_t)ucap * m->nblocks))) return st;
    if (lcap > 0 &&
        (st = ensure(c, m->llist, sizeof(uint16_t) * (size_t)lcap * kBlock * m->nblocks)))
        return st;
    if (lcap_leaf > 0 &&
        (st = ensure(c, m->llist_leaf, sizeof(uint16_t) * (size_t)lcap_leaf * m->nL)))
        return st;
    m->union_smem = sizeof(int32_t) * (2 * (size_t)fcap + p2);
    m->step_smem = sizeof(int4) * (size_t)m->ucap_sm * m->apl;
    m->lists_smpos = m->ucap_sm * m->apl;
    m->lists_smem = sizeof(float4) * (size_t)m->lists_smpos;
    // threads per atom of the step kernel: more than one for grids under two
    // waves of one block per SM, when the slice partials fit beside the
    // staged union
    {
        int nsm = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
        auto fits = [&](int t) {
            const size_t part_sm = sizeof(float) * 8 * kBlock * (size_t)(t - 1);
            return (int)(m->step_smem + part_sm) + 1024 <= maxsm;
        };
        const int req = m->p.threads_per_atom;
        if (m->nsys > 0) m->tpa = 1;
        else if (req > 0) m->tpa = fits(req) ? req : 1;
        else m->tpa = (m->nblocks < 2 * nsm && fits(kSmallTPA)) ? kSmallTPA : 1;
        // thread blocks per block of atoms with 4 threads per atom: the given
        // number, or (0) the most that keep the grid within one block per SM
        // (32,768 atoms: 128 blocks of 1,024 threads ran faster than 256 of 512)
        m->split = 1;
        if (m->tpa == kSmallTPA) {
            if (m->p.cta_split > 0) m->split = m->p.cta_split;
            else if (4 * m->nblocks <= nsm) m->split = 4;
            else if (2 * m->nblocks <= nsm) m->split = 2;
        }
    }
    if ((int)m->union_smem + 1024 > maxsm || (lcap > 0 && (int)m->step_smem + 1024 > maxsm)) {
        c->last_error = "neighbour union too large for shared memory";
        return ND_ERR_OVERFLOW;
    }
    // The dynamic shared-memory limit is a per-function, process-wide
    // attribute; every engine launches with its own size, so the limit is
    // raised once to the device maximum (less the function's static shared
    // memory) rather than set per engine.
    cudaError_t e = raise_smem_limit((const void*)k_md_block_union, maxsm);
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_block_lists<1>, maxsm);
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_block_lists<2>, maxsm);
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_block_lists<4>, maxsm);
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_block_lists<8>, maxsm);
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_block_lists<16>, maxsm);
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_block_lists<32>, maxsm);
#define ND_SMEM(C, MODE)                                                                        \
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_step<C, MODE, false>, maxsm);   \
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_step<C, MODE, true>, maxsm);    \
    if (e == cudaSuccess)                                                                       \
        e = raise_smem_limit((const void*)k_md_step<C, MODE, false, kSmallTPA>, maxsm);         \
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_step<C, MODE, false, 2>, maxsm);  \
    if (e == cudaSuccess)                                                                       \
        e = raise_smem_limit((const void*)k_md_step<C, MODE, false, kSmallTPA, 2>, maxsm);      \
    if (e == cudaSuccess)                                                                       \
        e = raise_smem_limit((const void*)k_md_step<C, MODE, false, kSmallTPA, 4>, maxsm);
    ND_SMEM(true, 0) ND_SMEM(false, 0) ND_SMEM(true, 1) ND_SMEM(false, 1) ND_SMEM(true, 2)
    ND_SMEM(false, 2) ND_SMEM(true, 3) ND_SMEM(false, 3)
#undef ND_SMEM
    if (e != cudaSuccess) return cuda_fail(c, e, "shared memory opt-in");
    return ND_OK;
}

StepArgs md_step_args(MDEngine* m, int rec_in) {
    StepArgs a{};
    const nd_md_params& p = m->p;
    a.n = m->n;
    a.apl = m->apl;
    a.ucap = m->ucap;
    a.lcap = m->lcap;
    a.smrec = m->ucap_sm * m->apl;
    a.ulist = (const int32_t*)m->ulist.p;
    a.ucount = (const int32_t*)m->ucount.p;
    a.llist = (const uint16_t*)m->llist.p;
    a.ncount = (const int32_t*)m->ncount.p;
    a.rec_in = (const int4*)m->rec_buf[rec_in].p;
    a.rec_out = (int4*)m->rec_buf[rec_in ^ 1].p;
    a.recf_in = (const uint2*)m->recf_buf[rec_in].p;
    a.recf_out = (uint2*)m->recf_buf[rec_in ^ 1].p;
    for (int d = 0; d < 3; ++d) {
        a.x[d] = m->set[m->cur].x[d];
        a.w[d] = m->set[m->cur].w[d];
        a.v_out[d] = (double*)m->vtmp.p + (size_t)d * m->n;
        a.lo[d] = p.box_lo[d];
        a.hi[d] = p.box_hi[d];
    }
    a.im = m->set[m->cur].im;
    a.f_out = (float4*)m->f.p;
    a.acc = (double*)m->acc.p;
    a.rec_build = (const int4*)m->recb.p;
    a.diag = (unsigned long long*)m->diag.p;
    a.err = m->sub.d_err;
    const double S = m->fr.s;
    // The lists are built from Float32 positions; a distance rounded there
    // errs by a few ulps of the largest coordinate, which the bound on the
    // displacement gives back.
    double cmax = 0.0;
    if (m->nsys > 0) cmax = m->tree_frame[3];
    else
        for (int d = 0; d < 3; ++d) cmax = std::max({cmax, std::fabs(p.box_lo[d]), std::fabs(p.box_hi[d])});
    const double ulp = std::ldexp(1.0, std::ilogb(std::max(cmax, 1.0)) - 23);
    const float hs = (float)(std::max(0.0, 0.5 * p.skin - 4.0 * ulp) * S);
    a.half_skin2u = hs * hs;
    a.hsu = hs;
    a.ctl = (unsigned*)m->ctl.p;
    a.cond = 0;
    a.use_cond = 0;
    a.vote = 1;
    a.trig_k = 2.0f * (float)std::max(m->check_every - 1, 1);
    a.unchecked = 0;
    for (int d = 0; d < 3; ++d) {
        a.os[d] = m->fr.o[d] * S * kFine;
        a.lo_fp[d] = (int64_t)std::floor((p.box_lo[d] - m->fr.o[d]) * S * kFine);
        a.hi_fp[d] = (int64_t)std::ceil((p.box_hi[d] - m->fr.o[d]) * S * kFine);
    }
    a.nk = md_near(p.sigma, p.epsilon, p.coulomb_k, p.cutoff, S);
    a.rc2u = (float)(p.cutoff * p.cutoff * S * S);
    a.sig2u = (float)(p.sigma * p.sigma * S * S);
    a.eps24u = (float)(24.0 * p.epsilon * S);
    a.eps4 = (float)(4.0 * p.epsilon);
    a.kcu = (float)(p.coulomb_k * S * S);
    a.kceu = (float)(p.coulomb_k * S);
    a.hdt = (float)(0.5 * p.dt);
    a.dt = p.dt;
    a.fr = m->fr;
    a.sid = m->set[m->cur].sid;
    a.sys = (const SysRow*)m->sysrow.p;
    a.nsys = m->nsys;
    return a;
}

template <int MODE>
static void launch_step_impl(MDEngine* m, const StepArgs& a0, bool first) {
    Ctx* c = &m->sub;
    const unsigned grid = (unsigned)m->nblocks;
    const size_t sm = m->step_smem;
    const bool coul = m->has_q && m->p.coulomb_k != 0.0;
    StepArgs a = a0;
    a.first = first ? 1 : 0;
    a.has_mass = m->has_m ? 1 : 0;
#define ND_STEP(BATCH, TPA, SPLIT)                                                              \
    do {                                                                                        \
        const unsigned gs = grid * SPLIT, bs = kBlock * TPA / SPLIT;                            \
        if (coul) k_md_step<true, MODE, BATCH, TPA, SPLIT><<<gs, bs, sm, c->stream>>>(a);       \
        else k_md_step<false, MODE, BATCH, TPA, SPLIT><<<gs, bs, sm, c->stream>>>(a);           \
    } while (0)
    if (m->nsys > 0) ND_STEP(true, 1, 1);
    else if (m->tpa == kSmallTPA && m->split == 4) ND_STEP(false, kSmallTPA, 4);
    else if (m->tpa == kSmallTPA && m->split == 2) ND_STEP(false, kSmallTPA, 2);
    else if (m->tpa == kSmallTPA) ND_STEP(false, kSmallTPA, 1);
    else if (m->tpa == 2) ND_STEP(false, 2, 1);
    else ND_STEP(false, 1, 1);
#undef ND_STEP
    c->launches++;
}

// MODE 0 steps inside a captured window publish their early-refit vote to the
// conditional node after them (MODE 2); the others are plain kernels.
template <int MODE>
static void launch_step(MDEngine* m, const StepArgs& a, bool first) {
    if (MODE == 0 && a.use_cond) launch_step_impl<2>(m, a, first);
    else launch_step_impl<MODE>(m, a, first);
}

void md_launch_step(MDEngine* m, const StepArgs& a, bool first) { launch_step<0>(m, a, first); }

// ctl words: [0] early-refit request, [1] finished-block tickets, [2] early
// refits done, [3] window counter, [4] capacity pressure, [5] rebuild
// decision, [6] re-sorts done, [7] scheduled refits done.
static unsigned* ctl_word(MDEngine* m, int k) { return (unsigned*)m->ctl.p + k; }

// Rebuild of the neighbour lists.
//   RB_RESORT: Float32 positions -> codes -> sort -> gather the state into the
//   scratch set and copy it back (the live set keeps its addresses) -> leaf
//   boxes -> build -> block unions -> per-atom lists.
//   RB_REFIT: keeps the order and the sorted codes (so the build reproduces
//   the topology) and refreshes positions, boxes, unions and lists.
// rec >= 0: a refit inside a window (early refit) whose records go to record
// buffer `rec`, the one the next step reads; otherwise records go to buffer 0
// and the step parity restarts.  counter: device count of this kind of
// rebuild (nullptr: not counted).  sizing: capacity-sizing pass.
nd_status md_rebuild(MDEngine* m, int kind, int rec, unsigned* counter, bool sizing) {
    NvtxRange nv(kind == RB_REFIT ? "nd md rebuild (refit)" : "nd md rebuild (re-sort)");
    Ctx* c = &m->sub;
    const int32_t n = m->n;
    const unsigned g = (unsigned)cdiv(n, 256);
    int32_t* codes = (int32_t*)c->codes.p;
    int32_t* perm = (int32_t*)c->perm.p;
    nd_status st;
    const SysRow* sys = (const SysRow*)m->sysrow.p;
    SetPtrs& live = m->set[0];
    // a new list answers any pending early-refit request
    if (cudaMemsetAsync(m->ctl.p, 0, 2 * sizeof(unsigned), c->stream) != cudaSuccess)
        return cuda_fail(c, cudaGetLastError(), "md rebuild");
    if (kind == RB_REFIT) {
        k_md_refit_pos<<<g, 256, 0, c->stream>>>(
            live, n, m->fr, sys, (float4*)m->pos32.p, (int4*)m->rec_buf[rec >= 0 ? rec : 0].p,
            (uint2*)m->recf_buf[rec >= 0 ? rec : 0].p, (int4*)m->recb.p, c->d_err, counter);
        c->launches++;
    } else {
        SetPtrs& tmp = m->set[1];
        k_md_pos32<<<g, 256, 0, c->stream>>>(live.x[0], live.x[1], live.x[2], live.sid, sys, n,
                                             (float*)m->xyz32.p, counter);
        c->launches++;
        // a batched ensemble sorts on the fixed slot grid, so every system is
        // one contiguous run of the Hilbert order
        if ((st = morton_codes(c, (const float*)m->xyz32.p, n, m->p.order, codes, perm,
                               m->nsys > 0 ? m->tree_frame : nullptr)))
            return st;
        if ((st = radix_sort_pairs(c, (uint32_t*)codes, perm, n, 30))) return st;
        k_md_reorder<<<g, 256, 0, c->stream>>>(live, tmp, perm, (const float*)m->xyz32.p, n,
                                               m->fr, sys, (float4*)m->pos32.p,
                                               (int4*)m->rec_buf[0].p, (uint2*)m->recf_buf[0].p,
                                               (int4*)m->recb.p, c->d_err);
        k_md_copy_set<<<g, 256, 0, c->stream>>>(tmp, live, n);
        c->launches += 2;
    }
    unsigned* pressure = sizing ? nullptr : ctl_word(m, 4);
    float4* keys = (float4*)m->keys.p;
    const float rl = (float)(m->p.cutoff + m->p.skin);
    k_md_leaf_boxes<<<(unsigned)cdiv(m->nL, 128), 128, 0, c->stream>>>(
        (const float4*)m->pos32.p, m->nL, m->apl, rl / 2.0f, keys);
    c->launches++;
    const bool tree = m->p.union_search == ND_UNION_TREE;
    if (tree) {
        if ((st = build_internal_nodes(c, keys, (int32_t*)m->store.p, codes, m->nL, m->apl)))
            return st;
    } else {
        k_md_block_boxes<<<(unsigned)cdiv(m->nblocks, 32), 1024, 0, c->stream>>>(
            keys, m->nL, m->nblocks, kBlock / m->apl, (float4*)m->bbox.p);
        c->launches++;
    }
    // query boxes slightly above r_list/2 so the box tests never drop a pair;
    // the distance test alone decides membership
    const float hq = (rl / 2.0f) * 1.0001f + 1e-6f;
    k_md_block_union<<<(unsigned)m->nblocks, kBlock, m->union_smem, c->stream>>>(
        keys, (const float4*)m->bbox.p, m->nblocks, tree ? 1 : 0, (const float4*)m->pos32.p,
        live.sid, n, m->nL, m->apl, hq, rl, m->fcap, m->ucap,
        m->upow2, (int32_t*)m->ulist.p, (int32_t*)m->ucount.p, (uint16_t*)m->llist_leaf.p,
        (int32_t*)m->lcount_leaf.p, m->lcap_leaf, c->d_err, (int32_t*)m->diag.p + 2,
        sizing ? 1 : 0, pressure);
#define ND_LISTS(A)                                                                             \
    k_md_block_lists<A><<<(unsigned)m->nblocks, kBlock, m->lists_smem, c->stream>>>(            \
        (const float4*)m->pos32.p, n, rl * rl,                                                  \
        md_near(m->p.sigma, m->p.epsilon, m->p.coulomb_k, m->p.cutoff, m->fr.s).rnb2,           \
        m->nsys > 0 ? live.sid : nullptr, sys, m->ucap, m->lists_smpos,                         \
        (const int32_t*)m->ulist.p, (const int32_t*)m->ucount.p,                                \
        (const uint16_t*)m->llist_leaf.p, (const int32_t*)m->lcount_leaf.p, m->lcap_leaf,       \
        m->lcap, (uint16_t*)m->llist.p, (int32_t*)m->ncount.p, c->d_err,                        \
        (int32_t*)m->diag.p + 2, sizing ? 1 : 0, pressure)
    switch (m->apl) {
        case 1: ND_LISTS(1); break;
        case 2: ND_LISTS(2); break;
        case 4: ND_LISTS(4); break;
        case 8: ND_LISTS(8); break;
        case 16: ND_LISTS(16); break;
        default: ND_LISTS(32); break;
    }
#undef ND_LISTS
    c->launches += 2;
    if (rec < 0) m->rc = 0;
    return check_launch(c, "md rebuild");
}

// Rebuild at the start of a window, re-sort or refit as k_md_window_begin
// decides on the device: inside a capture an IF/ELSE node, otherwise after
// reading the decision back.
static nd_status md_window_begin(MDEngine* m, bool capture) {
    NvtxRange nv("nd md window begin");
    Ctx* c = &m->sub;
    nd_status st;
    cudaGraphConditionalHandle h = 0;
    if (capture && (st = md_cond_handle(m, &h))) return st;
    k_md_window_begin<<<1, 32, 0, c->stream>>>((unsigned*)m->ctl.p, m->resort_every, h,
                                               capture ? 1 : 0);
    c->launches++;
    if (capture) {
        int64_t nk[2] = {0, 0};
        nd_status s2 = md_add_cond_node(
            m, h, 2,
            [&](int k) {
                return k == 0 ? md_rebuild(m, RB_RESORT, -1, ctl_word(m, 6))
                              : md_rebuild(m, RB_REFIT, -1, ctl_word(m, 7));
            },
            nk);
        if (s2 == ND_OK) { m->resort_kernels = nk[0]; m->refit_kernels = nk[1]; }
        return s2;
    }
    unsigned need = 0;
    cudaError_t e = cudaMemcpyAsync(&need, ctl_word(m, 5), sizeof(need), cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "rebuild decision");
    const int64_t l0 = c->launches;
    st = need ? md_rebuild(m, RB_RESORT, -1, ctl_word(m, 6))
              : md_rebuild(m, RB_REFIT, -1, ctl_word(m, 7));
    m->eager_bodies += c->launches - l0;
    return st;
}

// ---------------------------------------------------------- observers
// The step loop of simulate! (Simulator.jl:241-245) rescales the velocities
// every 10 steps (rescale_velocity!, :119-144) and appends the positions to
// its log after every step.  Here both are optional, run after the steps
// whose global index they divide, and inside captured windows are IF nodes
// whose conditions k_md_due sets from the device's window counter.

__global__ void k_md_due(const unsigned* __restrict__ ctl, int32_t R, int32_t p, int32_t every_t,
                         int32_t every_l, cudaGraphConditionalHandle ht,
                         cudaGraphConditionalHandle hl) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    // ctl[3] is the current window's number + 1
    const long long g = (long long)(ctl[3] - 1u) * R + p + 1;
    if (every_t > 0) cudaGraphSetConditional(ht, g % every_t == 0 ? 1u : 0u);
    if (every_l > 0) cudaGraphSetConditional(hl, g % every_l == 0 ? 1u : 0u);
}

// rescale_velocity!, 1: per block of 256 atoms the sum of |v_i| m_i / 2 over
// the integer-step velocities v (component-major, 3 x n), fixed order.
__global__ void __launch_bounds__(256) k_md_thermo_part(const double* __restrict__ v,
                                                        const double* __restrict__ im, int32_t n,
                                                        double* __restrict__ part) {
    __shared__ double s[256];
    const int32_t i = blockIdx.x * 256 + threadIdx.x;
    double t = 0.0;
    if (i < n) {
        const double a = v[i], b = v[(int64_t)n + i], c = v[2 * (int64_t)n + i];
        t = sqrt(a * a + b * b + c * c) / im[i] / 2.0;
    }
    s[threadIdx.x] = t;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// 2: Ti = 2 / (3 N kb) * sum (kb = 1), beta = (1 + gamma (Tf / Ti - 1))^0.5.
// Ti <= 0 keeps beta = 1; a negative radicand (the reference's DomainError)
// keeps beta = 1 and reports ND_ERR_ARG.  obs: [0] frames logged,
// [1] thermostat applications (uint64), [2] the last beta (double).
__global__ void k_md_thermo_beta(const double* __restrict__ part, int32_t nb, int32_t n,
                                 double Tf, double gamma, unsigned long long* obs, int32_t* err) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double sum = 0.0;
    for (int32_t b = 0; b < nb; ++b) sum += part[b];
    const double Ti = 2.0 / (3.0 * (double)n) * sum;
    double beta = 1.0;
    if (Ti > 0.0) {
        const double r = 1.0 + gamma * (Tf / Ti - 1.0);
        if (r >= 0.0) beta = sqrt(r);
        else set_error(err, ND_ERR_ARG, 0);
    }
    reinterpret_cast<double*>(obs)[2] = beta;
    obs[1] += 1ull;
}

// 3: v <- beta v on the half-step state: u = beta v - dt/2 F/m, so the next
// step's two half kicks continue from the rescaled integer-step velocity.
__global__ void k_md_thermo_scale(double* w0, double* w1, double* w2, const double* __restrict__ v,
                                  const float4* __restrict__ f, const double* __restrict__ im,
                                  int32_t n, float hdt, const unsigned long long* obs) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double beta = reinterpret_cast<const double*>(obs)[2];
    const float4 g = f[i];
    const double imv = im[i];
    w0[i] = beta * v[i] - (double)(hdt * g.x) * imv;
    w1[i] = beta * v[(int64_t)n + i] - (double)(hdt * g.y) * imv;
    w2[i] = beta * v[2 * (int64_t)n + i] - (double)(hdt * g.z) * imv;
}

// Position log: frame (frames logged mod ring size) <- positions in the
// caller's order; k_md_log_advance counts the frame afterwards.
__global__ void k_md_log(const double* __restrict__ x0, const double* __restrict__ x1,
                         const double* __restrict__ x2, const int32_t* __restrict__ orig, int32_t n,
                         double* __restrict__ ring, int64_t frames,
                         const unsigned long long* __restrict__ obs) {
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t slot = (int64_t)(obs[0] % (unsigned long long)frames);
    double* fr = ring + slot * 3 * (int64_t)n;
    const int64_t o = orig[k];
    fr[3 * o] = x0[k];
    fr[3 * o + 1] = x1[k];
    fr[3 * o + 2] = x2[k];
}

__global__ void k_md_log_advance(unsigned long long* obs) {
    if (threadIdx.x == 0 && blockIdx.x == 0) obs[0] += 1ull;
}

static nd_status md_thermo_body(MDEngine* m) {
    Ctx* c = &m->sub;
    const unsigned g = (unsigned)cdiv(m->n, 256);
    StepArgs a = md_step_args(m, m->rc);
    launch_step<3>(m, a, false);  // integer-step velocities and forces
    const double* vt = (const double*)m->vtmp.p;
    SetPtrs& s = m->set[0];
    k_md_thermo_part<<<g, 256, 0, c->stream>>>(vt, s.im, m->n, (double*)m->obs_part.p);
    k_md_thermo_beta<<<1, 32, 0, c->stream>>>((const double*)m->obs_part.p, (int32_t)g, m->n,
                                              m->thermo_T, m->thermo_gamma,
                                              (unsigned long long*)m->obs.p, c->d_err);
    k_md_thermo_scale<<<g, 256, 0, c->stream>>>(s.w[0], s.w[1], s.w[2], vt, (const float4*)m->f.p,
                                                s.im, m->n, (float)(0.5 * m->p.dt),
                                                (const unsigned long long*)m->obs.p);
    c->launches += 3;
    return check_launch(c, "thermostat");
}

static nd_status md_log_body(MDEngine* m) {
    Ctx* c = &m->sub;
    SetPtrs& s = m->set[0];
    k_md_log<<<(unsigned)cdiv(m->n, 256), 256, 0, c->stream>>>(
        s.x[0], s.x[1], s.x[2], s.orig, m->n, (double*)m->logbuf.p, m->log_frames,
        (const unsigned long long*)m->obs.p);
    k_md_log_advance<<<1, 32, 0, c->stream>>>((unsigned long long*)m->obs.p);
    c->launches += 2;
    return check_launch(c, "position log");
}

static int32_t gcd32(int32_t a, int32_t b) {
    while (b) { const int32_t t = a % b; a = b; b = t; }
    return a;
}

// Observers after the step at window position p (global step g on the host).
static nd_status md_observe(MDEngine* m, int32_t p, bool capture, int64_t g) {
    if (m->thermo_every <= 0 && m->log_every <= 0) return ND_OK;
    Ctx* c = &m->sub;
    const int32_t R = m->p.rebuild_every;
    auto possible = [&](int32_t every) { return every > 0 && (p + 1) % gcd32(every, R) == 0; };
    const bool pt = possible(m->thermo_every), pl = possible(m->log_every);
    if (!pt && !pl) return ND_OK;
    nd_status st;
    if (!capture) {
        const int64_t l0 = c->launches;
        if (pt && g % m->thermo_every == 0 && (st = md_thermo_body(m))) return st;
        if (pl && g % m->log_every == 0 && (st = md_log_body(m))) return st;
        m->eager_bodies += c->launches - l0;
        return ND_OK;
    }
    cudaGraphConditionalHandle ht = 0, hl = 0;
    if (pt && (st = md_cond_handle(m, &ht))) return st;
    if (pl && (st = md_cond_handle(m, &hl))) return st;
    k_md_due<<<1, 32, 0, c->stream>>>((const unsigned*)m->ctl.p, R, p, pt ? m->thermo_every : 0,
                                      pl ? m->log_every : 0, ht, hl);
    c->launches++;
    if (pt && (st = md_add_cond_node(m, ht, 1, [&](int) { return md_thermo_body(m); },
                                     &m->thermo_kernels)))
        return st;
    if (pl && (st = md_add_cond_node(m, hl, 1, [&](int) { return md_log_body(m); },
                                     &m->log_kernels)))
        return st;
    return ND_OK;
}

// Enqueue `k` steps of the current window, the first at window position pos0.
// After the window's steps 0, M, 2M, ... (M = check_every) but not its last, a
// refit runs if some atom could pass skin/2 from its list-build position
// before the next check: inside a capture as a conditional node (one handle
// per node, set by the step before it), otherwise eagerly after reading the
// request flag.  ev (eager only): a pair
// of events per step recorded around the step kernel.
static nd_status md_steps(MDEngine* m, int32_t k, int32_t pos0, bool capture = false,
                          cudaEvent_t* ev = nullptr) {
    NvtxRange nv(capture ? "nd md capture steps" : "nd md steps");
    Ctx* c = &m->sub;
    const int32_t R = m->p.rebuild_every;
    nd_status st;
    for (int32_t s = 0; s < k; ++s) {
        // a check follows the window's steps 0, M, 2M, ... but not its last
        const int32_t p = (pos0 + s) % R;
        const bool check = p != R - 1 && p % m->check_every == 0;
        cudaGraphConditionalHandle h = 0;
        if (capture && check && (st = md_cond_handle(m, &h))) return st;
        StepArgs a = md_step_args(m, m->rc);
        a.use_cond = capture && check ? 1 : 0;
        a.vote = check ? 1 : 0;
        a.unchecked = !check && p != R - 1 ? 1 : 0;
        a.cond = h;
        if (ev) cudaEventRecord(ev[2 * s], c->stream);
        launch_step<0>(m, a, m->first);
        if (ev) cudaEventRecord(ev[2 * s + 1], c->stream);
        m->first = false;
        m->rc ^= 1;
        if (check && capture) {
            if ((st = md_add_cond_node(
                     m, h, 1, [&](int) { return md_rebuild(m, RB_REFIT, m->rc, ctl_word(m, 2)); },
                     &m->refit_kernels)))
                return st;
        } else if (check) {
            unsigned flag = 0;
            cudaError_t e = cudaMemcpyAsync(&flag, m->ctl.p, sizeof(flag), cudaMemcpyDeviceToHost,
                                            c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "refit request");
            if (flag) {
                const int64_t l0 = c->launches;
                if ((st = md_rebuild(m, RB_REFIT, m->rc, ctl_word(m, 2)))) return st;
                m->eager_bodies += c->launches - l0;
            }
        }
        if ((st = md_observe(m, pos0 + s, capture, m->steps + s + 1))) return st;
    }
    return ND_OK;
}

// The opening window after an upload (no rebuild: the upload built the list;
// its first step completes only a half kick).
static nd_status md_capture_first(MDEngine* m) {
    Ctx* c = &m->sub;
    const int save_rc = m->rc;
    const bool save_first = m->first;
    const int64_t save_launch = c->launches;
    m->first = true;
    m->rc = 0;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(c, e, "begin capture");
    nd_status st = md_steps(m, m->p.rebuild_every, 0, true);
    e = cudaStreamEndCapture(c->stream, &g);
    if (st) { if (g) cudaGraphDestroy(g); return st; }
    if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
    e = cudaGraphInstantiate(&m->graph_first, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "graph instantiate");
    m->graph_first_launches = c->launches - save_launch;
    c->launches = save_launch;
    m->rc = save_rc;
    m->first = save_first;
    return ND_OK;
}

// Every later window: device-decided rebuild + R steps.
static nd_status md_capture_main(MDEngine* m) {
    Ctx* c = &m->sub;
    const int save_rc = m->rc;
    const bool save_first = m->first;
    const int64_t save_launch = c->launches;
    m->first = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(c, e, "begin capture");
    nd_status st = md_window_begin(m, true);
    if (st == ND_OK) st = md_steps(m, m->p.rebuild_every, 0, true);
    e = cudaStreamEndCapture(c->stream, &g);
    if (st) { if (g) cudaGraphDestroy(g); return st; }
    if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
    e = cudaGraphInstantiate(&m->graph_main, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "graph instantiate");
    m->graph_main_launches = c->launches - save_launch;
    c->launches = save_launch;
    m->rc = save_rc;
    m->first = save_first;
    return ND_OK;
}

// Window counter after an opening build: that build was window 0.
static nd_status md_opened(MDEngine* m) {
    const unsigned one = 1u;
    cudaError_t e = cudaMemcpyAsync(ctl_word(m, 3), &one, sizeof(one), cudaMemcpyHostToDevice,
                                    m->sub.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->sub.stream);
    if (e != cudaSuccess) return cuda_fail(&m->sub, e, "window counter");
    return ND_OK;
}

// Sizing build pass: diag int32 words 2..6 collect the largest union, the
// largest per-atom list, the largest per-leaf candidate list, the sum of
// union sizes and the largest BFS frontier.
static nd_status md_sizing_pass(MDEngine* m, int32_t h[5]) {
    Ctx* c = &m->sub;
    cudaMemsetAsync((int32_t*)m->diag.p + 2, 0, 5 * sizeof(int32_t), c->stream);
    nd_status st = md_rebuild(m, RB_RESORT, -1, nullptr, true);
    if (st) return st;
    cudaError_t e = cudaMemcpyAsync(h, (int32_t*)m->diag.p + 2, 5 * sizeof(int32_t),
                                    cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "size lists");
    return sync_and_check(c, "md sizing build");
}

static int32_t round_up(double v, int32_t q) { return (((int32_t)std::ceil(v)) + q - 1) / q * q; }

// First builds: (1) generous union and frontier, lists not stored -> union,
// frontier and per-leaf capacities; (2) per-leaf lists stored, per-atom lists
// counted -> list capacity; (3) the real build.  Capacities carry head-room
// for the drift until later rebuilds.
static nd_status md_size_lists(MDEngine* m) {
    Ctx* c = &m->sub;
    nd_status st;
    int32_t h[5];
    if ((st = md_alloc_lists(m, kSizingFcap, kSizingUcap, 0, 0, 0))) return st;
    if ((st = md_sizing_pass(m, h))) return st;
    const int32_t max_u = h[0], max_c = h[2], max_f = h[4];
    const double mean_u = (double)h[3] / m->nblocks;
    if (max_u > kSizingUcap || max_f > kSizingFcap) {
        c->last_error = "neighbour union of a block exceeds the supported size";
        return ND_ERR_OVERFLOW;
    }
    int32_t ucap = round_up(max_u * 1.25 + 32, 32);
    if ((int64_t)ucap * m->apl > 65536) ucap = 65536 / m->apl;
    const int32_t fcap = round_up(max_f * 1.3 + 64, 32);
    const int32_t lcap_leaf = std::min(ucap, round_up(max_c * 1.3 + 16, 8));
    // Shared-memory staging sized near the mean union (head-room for drift);
    // a block whose union is larger reads its remaining records from L2.
    const int32_t ucap_sm = m->p.stage_policy == 1 ? ucap : round_up(mean_u * 1.2 + 16, 16);
    if ((st = md_alloc_lists(m, fcap, ucap, lcap_leaf, 0, ucap_sm))) return st;
    if ((st = md_sizing_pass(m, h))) return st;
    const int32_t max_n = h[1];
    int32_t lcap = m->p.max_neighbors > 0 ? round_up(m->p.max_neighbors, 8)
                                          : round_up(max_n * 1.35 + 16, 8);
    if ((st = md_alloc_lists(m, fcap, ucap, lcap_leaf, lcap, ucap_sm))) return st;
    if ((st = md_rebuild(m, RB_RESORT))) return st;
    if ((st = md_opened(m))) return st;
    m->in_window = 0;
    m->rebuild_due = false;
    m->rebuilds = 1;
    return sync_and_check(c, "md first build");
}

nd_status md_destroy(MDEngine* m);

// Copy x, v (N x 3), q, m (N) from host or device memory into state set 0 in
// the caller's order and reset the step bookkeeping.
nd_status md_upload(MDEngine* m, const double* xd, const double* vd, const double* qd,
                    const double* md_, bool host) {
    Ctx* c = &m->sub;
    const int32_t n = m->n;
    const size_t bytes = 3 * sizeof(double) * (size_t)n;
    nd_status st;
    if ((st = ensure(c, m->aos, 2 * bytes + 2 * sizeof(double) * (size_t)n))) return st;
    double* ax = (double*)m->aos.p;
    double* av = ax + 3 * (size_t)n;
    double* aq = av + 3 * (size_t)n;
    double* am = aq + (size_t)n;
    cudaMemcpyKind kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpyAsync(ax, xd, bytes, kind, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(av, vd, bytes, kind, c->stream);
    if (e == cudaSuccess && qd) e = cudaMemcpyAsync(aq, qd, sizeof(double) * n, kind, c->stream);
    if (e == cudaSuccess && md_) e = cudaMemcpyAsync(am, md_, sizeof(double) * n, kind, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "md upload");
    const unsigned g = (unsigned)cdiv(n, 256);
    SetPtrs& s = m->set[0];
    k_md_split_aos<<<g, 256, 0, c->stream>>>(ax, n, s.x[0], s.x[1], s.x[2]);
    k_md_split_aos<<<g, 256, 0, c->stream>>>(av, n, s.w[0], s.w[1], s.w[2]);
    k_md_init_scalars<<<g, 256, 0, c->stream>>>(qd ? aq : nullptr, md_ ? am : nullptr,
                                                (const int32_t*)m->sid_in.p, n, s.q, s.im,
                                                s.orig, s.sid);
    c->launches += 3;
    if (cudaMemsetAsync(m->diag.p, 0, 64, c->stream) != cudaSuccess) return ND_ERR_CUDA;
    if (cudaMemsetAsync(m->ctl.p, 0, 64, c->stream) != cudaSuccess) return ND_ERR_CUDA;
    if (m->obs.p && cudaMemsetAsync(m->obs.p, 0, 64, c->stream) != cudaSuccess) return ND_ERR_CUDA;
    m->cur = 0;
    m->first = true;
    m->steps = 0;
    m->rebuilds = 0;
    m->in_window = 0;
    m->rebuild_due = false;
    return check_launch(c, "md upload");
}

// Re-use an engine (buffers, captured graphs) for a new state of the same
// size and parameters: upload, then the opening rebuild with the current list
// capacities.  ND_ERR_OVERFLOW means the caller must create a new engine.
nd_status md_reset(MDEngine* m, const double* x, const double* v, const double* q,
                   const double* mass, bool host) {
    if ((q != nullptr) != m->has_q || (mass != nullptr) != m->has_m) return ND_ERR_ARG;
    nd_status st = md_upload(m, x, v, q, mass, host);
    if (st) return st;
    if ((st = md_rebuild(m, RB_RESORT))) return st;
    if ((st = md_opened(m))) return st;
    m->rebuilds = 1;
    return sync_and_check(&m->sub, "md reset");
}

bool md_compatible(MDEngine* m, const nd_md_params* p, int32_t n, bool has_q, bool has_m) {
    return m && m->n == n && m->has_q == has_q && m->has_m == has_m &&
           memcmp(&m->p, p, sizeof(nd_md_params)) == 0;
}

// Fixed-point frame from the walls: origin 1/16 of the largest extent below
// the lower walls, scale from md_scale.
static nd_status md_frame(MDEngine* m) {
    double ext = 0.0;
    for (int d = 0; d < 3; ++d) ext = std::max(ext, m->p.box_hi[d] - m->p.box_lo[d]);
    if (!(ext > 0.0) || !std::isfinite(ext)) return ND_ERR_ARG;
    const double margin = ext / 16.0;
    for (int d = 0; d < 3; ++d) m->fr.o[d] = m->p.box_lo[d] - margin;
    m->fr.s = md_scale(m->p);
    m->fr.lim = md_frame_lim(ext, m->fr.s);
    return ND_OK;
}

// Batched ensemble frames.  Slots: a G x G x G grid (G a power of two, G^3 >=
// nsys) of cubes of side (largest system extent + 2 r_list + 1), system s in
// slot (s mod G, s/G mod G, s/G^2) with half the gap on every side.  The
// Hilbert grid spans the slot grid exactly, so each slot is one aligned
// sub-cube of the curve and each system one contiguous run of the order.
// Fixed point: per-system origin (walls less 1/16 of the extent), one scale.
static nd_status md_frame_batch(MDEngine* m, const nd_system* sys) {
    const int32_t ns = m->nsys;
    double side_max = 0.0;
    for (int32_t k = 0; k < ns; ++k)
        for (int d = 0; d < 3; ++d) {
            const double e = sys[k].box_hi[d] - sys[k].box_lo[d];
            if (!(e > 0.0) || !std::isfinite(e)) return ND_ERR_ARG;
            side_max = std::max(side_max, e);
        }
    const double rl = m->p.cutoff + m->p.skin;
    const double gap = 2.0 * rl + 1.0;
    const double slot = side_max + gap;
    int32_t G = 1;
    while ((int64_t)G * G * G < ns) G *= 2;
    if (G > 1024) return ND_ERR_ARG;
    for (int d = 0; d < 3; ++d) { m->tree_frame[d] = 0.0f; m->tree_frame[3 + d] = (float)(G * slot); }
    m->fr.s = 1.0;  // unused: every system has its own scale
    for (int d = 0; d < 3; ++d) m->fr.o[d] = 0.0;
    // the lists come from Float32 tree-frame positions: give back a few ulps
    // of the largest coordinate from the displacement bound
    const double ulp = std::ldexp(1.0, std::ilogb(std::max((double)m->tree_frame[3], 1.0)) - 23);
    const double hs_phys = std::max(0.0, 0.5 * m->p.skin - 4.0 * ulp);
    std::vector<SysRow> rows(ns);
    for (int32_t k = 0; k < ns; ++k) {
        const nd_system& y = sys[k];
        if (!std::isfinite(y.sigma) || !std::isfinite(y.epsilon) || !(y.sigma > 0)) return ND_ERR_ARG;
        SysRow& r = rows[k];
        const int32_t cell[3] = {k % G, (k / G) % G, k / (G * G)};
        double ext = 0.0;
        for (int d = 0; d < 3; ++d) ext = std::max(ext, y.box_hi[d] - y.box_lo[d]);
        const double S = md_scale(m->p);
        r.s = S;
        r.lim = md_frame_lim(ext, S);
        for (int d = 0; d < 3; ++d) {
            r.o[d] = y.box_lo[d] - ext / 16.0;
            r.os[d] = r.o[d] * S * kFine;
            r.off[d] = cell[d] * slot + 0.5 * gap - y.box_lo[d];
            r.lo[d] = y.box_lo[d];
            r.hi[d] = y.box_hi[d];
            r.lo_fp[d] = (int64_t)std::floor((y.box_lo[d] - r.o[d]) * S * kFine);
            r.hi_fp[d] = (int64_t)std::ceil((y.box_hi[d] - r.o[d]) * S * kFine);
        }
        r.nk = md_near(y.sigma, y.epsilon, m->p.coulomb_k, m->p.cutoff, S);
        r.sig2u = (float)(y.sigma * y.sigma * S * S);
        r.eps24u = (float)(24.0 * y.epsilon * S);
        r.eps4 = (float)(4.0 * y.epsilon);
        r.rc2u = (float)(m->p.cutoff * m->p.cutoff * S * S);
        r.kcu = (float)(m->p.coulomb_k * S * S);
        r.kceu = (float)(m->p.coulomb_k * S);
        r.hsu = (float)(hs_phys * S);
        r.hs2u = r.hsu * r.hsu;
    }
    Ctx* c = &m->sub;
    nd_status st = ensure(c, m->sysrow, sizeof(SysRow) * (size_t)ns);
    if (st) return st;
    std::vector<int32_t> sid(m->n);
    int64_t at = 0;
    for (int32_t k = 0; k < ns; ++k)
        for (int32_t j = 0; j < sys[k].n_atoms; ++j) sid[at++] = k;
    if ((st = ensure(c, m->sid_in, sizeof(int32_t) * (size_t)m->n))) return st;
    cudaError_t e = cudaMemcpy(m->sysrow.p, rows.data(), sizeof(SysRow) * (size_t)ns,
                               cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(m->sid_in.p, sid.data(), sizeof(int32_t) * (size_t)m->n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(c, e, "batch tables");
    return ND_OK;
}

static nd_status md_create_common(Ctx* parent, const nd_md_params* p, int32_t n,
                                  const double* xd, const double* vd, const double* qd,
                                  const double* md_, bool host, bool capture, MDEngine** out,
                                  int32_t nsys = 0, const nd_system* sys = nullptr) {
    if (!parent || !p || !out || !xd || !vd || n <= 0) return ND_ERR_ARG;
    if (p->atomsperleaf <= 0 || n % p->atomsperleaf || n / p->atomsperleaf < 2) return ND_ERR_SPEC;
    if (32 % p->atomsperleaf != 0) return ND_ERR_SPEC;  // a warp holds whole leaves
    if (p->rebuild_every <= 0 || !(p->cutoff > 0) || !(p->skin >= 0) || !(p->dt > 0) ||
        p->resort_every < 0 || p->stage_policy < 0 || p->stage_policy > 1 ||
        (p->union_search != ND_UNION_BLOCKS && p->union_search != ND_UNION_TREE) ||
        p->refit_check_every < 0 ||
        (p->threads_per_atom != 0 && p->threads_per_atom != 1 && p->threads_per_atom != 2 &&
         p->threads_per_atom != kSmallTPA) ||
        (p->cta_split != 0 && p->cta_split != 1 && p->cta_split != 2 && p->cta_split != 4))
        return ND_ERR_ARG;
    if (nsys < 0 || (nsys > 0 && !sys)) return ND_ERR_ARG;
    if (nsys > 0) {
        int64_t tot = 0;
        for (int32_t k = 0; k < nsys; ++k) {
            // a leaf never spans two systems
            if (sys[k].n_atoms <= 0 || sys[k].n_atoms % p->atomsperleaf) return ND_ERR_SPEC;
            tot += sys[k].n_atoms;
        }
        if (tot != n) return ND_ERR_ARG;
    }
    MDEngine* m = new MDEngine();
    m->nsys = nsys;
    m->resort_every = p->resort_every > 0 ? p->resort_every : 1;
    m->check_every = p->refit_check_every > 0 ? p->refit_check_every : 1;
    m->parent = parent;
    m->sub.device = parent->device;
    m->sub.stream = parent->stream;
    m->sub.d_err = parent->d_err;
    m->sub.h_err = parent->h_err;
    m->p = *p;
    m->n = n;
    m->apl = p->atomsperleaf;
    m->nL = n / m->apl;
    m->nblocks = (int32_t)cdiv(n, kBlock);
    m->has_q = qd != nullptr;
    m->has_m = md_ != nullptr;
    nd_status st = nsys > 0 ? md_frame_batch(m, sys) : md_frame(m);
    if (st == ND_OK) st = md_alloc(m);
    if (st) { parent->last_error = m->sub.last_error; md_destroy(m); return st; }
    Ctx* c = &m->sub;
    if ((st = md_upload(m, xd, vd, qd, md_, host))) { parent->last_error = c->last_error; md_destroy(m); return st; }
    m->cur = 0;
    m->first = true;
    if ((st = md_size_lists(m))) { parent->last_error = c->last_error; md_destroy(m); return st; }
    if (capture && cudaStreamCreateWithFlags(&m->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        st = cuda_fail(c, cudaGetLastError(), "capture stream");
        parent->last_error = c->last_error;
        md_destroy(m);
        return st;
    }
    if (capture && ((st = md_capture_main(m)) || (st = md_capture_first(m)))) {
        parent->last_error = c->last_error;
        md_destroy(m);
        return st;
    }
    parent->launches += c->launches;
    c->launches = 0;
    *out = m;
    return ND_OK;
}

nd_status md_create(Ctx* parent, const nd_md_params* p, int32_t n, const double* x,
                    const double* v, const double* q, const double* mass, bool host,
                    bool capture, MDEngine** out) {
    NvtxRange nv("nd md create");
    return md_create_common(parent, p, n, x, v, q, mass, host, capture, out);
}

nd_status md_create_batch(Ctx* parent, const nd_md_params* p, int32_t nsys, const nd_system* sys,
                          const double* x, const double* v, const double* q, const double* mass,
                          bool host, MDEngine** out) {
    if (nsys <= 0 || !sys) return ND_ERR_ARG;
    int64_t n = 0;
    for (int32_t k = 0; k < nsys; ++k) n += std::max(sys[k].n_atoms, 0);
    if (n <= 0 || n > INT32_MAX) return ND_ERR_ARG;
    return md_create_common(parent, p, (int32_t)n, x, v, q, mass, host, true, out, nsys, sys);
}

// Autotuner.  Each candidate setting runs on a fresh engine from the same
// host state -- one untimed window, then trial_steps timed with events on the
// stream, early refits included -- and the settings are tuned one at a time
// (coordinate descent): skin (the given one and -0.2 .. +0.2 in steps of
// 0.1, not below kMinTunedSkin: a longer list against fewer early refits),
// atoms per leaf (the leaf and traversal width), re-sort interval,
// shared-memory staging policy, union search, early-refit check interval,
// threads per atom and thread blocks per block of atoms (single systems).
// Candidates that do not fit
// (shared memory, leaf size not dividing every system) are skipped.
nd_status md_autotune(Ctx* parent, const nd_md_params* p, int32_t n, int32_t nsys,
                      const nd_system* sys, const double* x, const double* v, const double* q,
                      const double* mass, int32_t trial_steps, nd_md_params* best,
                      double* sps) {
    if (!parent || !p || !best || trial_steps <= 0 || n <= 0) return ND_ERR_ARG;
    const int32_t R = std::max(p->rebuild_every, 1);
    const int64_t steps = ((int64_t)trial_steps + R - 1) / R * R;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return cuda_fail(parent, cudaGetLastError(), "autotune events");
    }
    // time one setting: seconds per step, < 0 when it does not fit
    auto trial = [&](const nd_md_params& c, double* t) -> nd_status {
        *t = -1.0;
        bool fits = c.atomsperleaf > 0 && 32 % c.atomsperleaf == 0 && n % c.atomsperleaf == 0 &&
                    n / c.atomsperleaf >= 2;
        for (int32_t k = 0; fits && k < nsys; ++k) fits = sys[k].n_atoms % c.atomsperleaf == 0;
        if (!fits) return ND_OK;
        MDEngine* m = nullptr;
        nd_status st = nsys > 0 ? md_create_batch(parent, &c, nsys, sys, x, v, q, mass, true, &m)
                                : md_create(parent, &c, n, x, v, q, mass, true, true, &m);
        if (st == ND_ERR_OVERFLOW) { parent->last_error.clear(); return ND_OK; }
        if (st) return st;
        st = md_run(m, R);
        if (st == ND_OK) st = md_sync(m);
        if (st == ND_OK) {
            cudaEventRecord(e0, m->sub.stream);
            st = md_run(m, steps);
            cudaEventRecord(e1, m->sub.stream);
            if (st == ND_OK) st = md_sync(m);
        }
        float ms = 0.0f;
        if (st == ND_OK && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess)
            *t = ms * 1e-3 / (double)steps;
        md_destroy(m);
        // a setting whose lists outgrow their capacities in the trial is not
        // a candidate (refit windows on a fast-changing system)
        if (st == ND_ERR_OVERFLOW) { parent->last_error.clear(); return ND_OK; }
        return st;
    };
    nd_md_params win = *p;
    if (win.resort_every <= 0) win.resort_every = 1;
    double best_t = -1.0;
    nd_status result = ND_OK;
    auto consider = [&](const nd_md_params& c) -> nd_status {
        double t = -1.0;
        nd_status st = trial(c, &t);
        if (st == ND_OK && t > 0.0 && (best_t < 0.0 || t < best_t)) { best_t = t; win = c; }
        return st;
    };
    {
        // a starting leaf size that fits
        const int32_t apls[] = {4, 2, 8, 1};
        for (int32_t a : apls) {
            nd_md_params c = win;
            c.atomsperleaf = a;
            if ((result = consider(c))) goto done;
            if (best_t > 0.0) break;
        }
        if (best_t < 0.0) { result = ND_ERR_SPEC; parent->last_error = "no autotune candidate fits"; goto done; }
        const nd_md_params start = win;
        for (double ds : {-0.2, -0.1, 0.1, 0.2}) {
            nd_md_params c = start;
            c.skin = p->skin + ds;
            if (c.skin < kMinTunedSkin - 1e-9) continue;
            if ((result = consider(c))) goto done;
        }
        const nd_md_params s1 = win;
        for (int32_t a : {2, 4, 8}) {
            if (a == s1.atomsperleaf) continue;
            nd_md_params c = s1;
            c.atomsperleaf = a;
            if ((result = consider(c))) goto done;
        }
        const nd_md_params s2 = win;
        for (int32_t rs : {1, 5, 10}) {
            if (rs == s2.resort_every) continue;
            nd_md_params c = s2;
            c.resort_every = rs;
            if ((result = consider(c))) goto done;
        }
        const nd_md_params s3 = win;
        nd_md_params c = s3;
        c.stage_policy = 1 - s3.stage_policy;
        if ((result = consider(c))) goto done;
        const nd_md_params s4 = win;
        c = s4;
        c.union_search = s4.union_search == ND_UNION_TREE ? ND_UNION_BLOCKS : ND_UNION_TREE;
        if ((result = consider(c))) goto done;
        const nd_md_params s5 = win;
        for (int32_t ce : {1, 2, 3}) {
            if (ce == std::max(s5.refit_check_every, 1)) continue;
            c = s5;
            c.refit_check_every = ce;
            if ((result = consider(c))) goto done;
        }
        // threads sharing an atom's list in the step kernel (single systems):
        // the fastest explicit value, so the result names the one it runs
        if (nsys == 0) {
            const nd_md_params s6 = win;
            double tbest = -1.0;
            for (int32_t t : {1, 2, kSmallTPA}) {
                c = s6;
                c.threads_per_atom = t;
                c.cta_split = 1;
                double tt = -1.0;
                if ((result = trial(c, &tt))) goto done;
                if (tt > 0.0 && (tbest < 0.0 || tt < tbest)) { tbest = tt; win = c; }
            }
            // with 4 threads per atom, the thread blocks per block of atoms
            if (win.threads_per_atom == kSmallTPA) {
                const nd_md_params s7 = win;
                for (int32_t sp : {2, 4}) {
                    c = s7;
                    c.cta_split = sp;
                    double tt = -1.0;
                    if ((result = trial(c, &tt))) goto done;
                    if (tt > 0.0 && (tbest < 0.0 || tt < tbest)) { tbest = tt; win = c; }
                }
            }
            if (tbest > 0.0) best_t = tbest;
        }
    }
done:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (result == ND_OK) {
        *best = win;
        if (sps) *sps = best_t;
    }
    return result;
}

nd_status md_destroy(MDEngine* m) {
    if (!m) return ND_OK;
    if (m->graph_main) cudaGraphExecDestroy(m->graph_main);
    if (m->graph_first) cudaGraphExecDestroy(m->graph_first);
    DevBuf* bufs[] = {&m->set_buf[0], &m->set_buf[1], &m->rec_buf[0], &m->rec_buf[1],
                      &m->recf_buf[0], &m->recf_buf[1], &m->recb,
                      &m->xyz32, &m->pos32, &m->keys, &m->store, &m->bbox, &m->ulist, &m->ucount,
                      &m->llist_leaf, &m->lcount_leaf, &m->llist,
                      &m->ncount, &m->f, &m->vtmp, &m->acc, &m->aos, &m->diag, &m->sysrow,
                      &m->sid_in, &m->ctl, &m->obs, &m->obs_part, &m->logbuf, &m->sub.codes,
                      &m->sub.codes_alt, &m->sub.perm, &m->sub.perm_alt, &m->sub.hist,
                      &m->sub.misc};
    if (m->sub.stream) cudaStreamSynchronize(m->sub.stream);
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    if (m->cap_stream) cudaStreamDestroy(m->cap_stream);
    delete m;
    return ND_OK;
}

// Advance `steps` steps: whole windows replay the captured graph of the
// current state set (rebuild + R steps); partial windows are enqueued eagerly.
nd_status md_run(MDEngine* m, int64_t steps) {
    NvtxRange nv("nd md run");
    Ctx* c = &m->sub;
    const int32_t R = m->p.rebuild_every;
    nd_status st;
    while (steps > 0) {
        if (m->rebuild_due) {
            if (steps >= R && !m->first && m->graph_main) {
                // a whole window: rebuild (decided on the device) + R steps
                cudaError_t e = cudaGraphLaunch(m->graph_main, c->stream);
                if (e != cudaSuccess) return cuda_fail(c, e, "graph launch");
                c->launches += m->graph_main_launches;
                m->rc = R & 1;
                m->rebuilds++;
                m->steps += R;
                steps -= R;
                continue;
            }
            if ((st = md_window_begin(m, false))) return st;
            m->rebuilds++;
            m->rebuild_due = false;
            m->in_window = 0;
        }
        if (m->first && m->in_window == 0 && steps >= R && m->graph_first) {
            // the opening window after an upload
            cudaError_t e = cudaGraphLaunch(m->graph_first, c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "graph launch");
            c->launches += m->graph_first_launches;
            m->first = false;
            m->rc = R & 1;
            m->rebuild_due = true;
            m->steps += R;
            steps -= R;
            continue;
        }
        int32_t k = (int32_t)std::min<int64_t>(steps, R - m->in_window);
        if ((st = md_steps(m, k, m->in_window))) return st;
        m->in_window += k;
        if (m->in_window == R) { m->in_window = 0; m->rebuild_due = true; }
        m->steps += k;
        steps -= k;
    }
    m->parent->launches += c->launches;
    c->launches = 0;
    return check_launch(c, "md run");
}

// Advance `steps` steps eagerly (rebuilds and early refits as usual), timing
// every step kernel with its own pair of events on the stream: ms[k] is the
// k-th step kernel's duration.
nd_status md_step_times(MDEngine* m, int32_t steps, float* ms) {
    NvtxRange nv("nd md step times");
    Ctx* c = &m->sub;
    if (steps <= 0 || !ms) return ND_ERR_ARG;
    const int32_t R = m->p.rebuild_every;
    std::vector<cudaEvent_t> ev(2 * (size_t)steps, nullptr);
    nd_status st = ND_OK;
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) { st = cuda_fail(c, cudaGetLastError(), "events"); break; }
    int32_t done = 0;
    while (st == ND_OK && done < steps) {
        if (m->rebuild_due) {
            if ((st = md_window_begin(m, false))) break;
            m->rebuilds++;
            m->rebuild_due = false;
            m->in_window = 0;
        }
        const int32_t k = std::min(steps - done, R - m->in_window);
        if ((st = md_steps(m, k, m->in_window, false, ev.data() + 2 * (size_t)done))) break;
        m->in_window += k;
        if (m->in_window == R) { m->in_window = 0; m->rebuild_due = true; }
        m->steps += k;
        done += k;
    }
    if (st == ND_OK) st = sync_and_check(c, "md step times");
    for (int32_t k = 0; st == ND_OK && k < steps; ++k) {
        cudaError_t e = cudaEventElapsedTime(&ms[k], ev[2 * k], ev[2 * k + 1]);
        if (e != cudaSuccess) st = cuda_fail(c, e, "event time");
    }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    m->parent->launches += c->launches;
    c->launches = 0;
    return st;
}

nd_status md_measure(MDEngine* m, bool energy) {
    Ctx* c = &m->sub;
    cudaMemsetAsync(m->acc.p, 0, 2 * sizeof(double) * (size_t)std::max(m->nsys, 1), c->stream);
    StepArgs a = md_step_args(m, m->rc);
    if (energy) launch_step<1>(m, a, m->first);
    else launch_step<3>(m, a, m->first);
    return check_launch(c, "md measure");
}

nd_status md_get(MDEngine* m, double* x, double* v, float* f, bool host) {
    Ctx* c = &m->sub;
    nd_status st = md_measure(m, false);
    if (st) return st;
    const size_t bytes = 3 * sizeof(double) * (size_t)m->n;
    double *dx = nullptr, *dv = nullptr;
    float* df = nullptr;
    if (host) {
        // stage through the AoS buffer (2 x 3N doubles) and the f32 tmp area
        if ((st = ensure(c, m->aos, 2 * bytes + 3 * sizeof(float) * (size_t)m->n))) return st;
        dx = (double*)m->aos.p;
        dv = dx + 3 * (size_t)m->n;
        df = (float*)(dv + 3 * (size_t)m->n);
    } else {
        dx = x; dv = v; df = f;
    }
    SetPtrs& s = m->set[m->cur];
    const double* vt = (const double*)m->vtmp.p;
    k_md_unsort<<<(unsigned)cdiv(m->n, 256), 256, 0, c->stream>>>(
        s.orig, m->n, s.x[0], s.x[1], s.x[2], vt, vt + m->n, vt + 2 * (size_t)m->n,
        (const float4*)m->f.p, x ? dx : nullptr, v ? dv : nullptr, f ? df : nullptr);
    c->launches++;
    if (host) {
        cudaError_t e = cudaSuccess;
        if (x) e = cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && v) e = cudaMemcpyAsync(v, dv, bytes, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && f)
            e = cudaMemcpyAsync(f, df, 3 * sizeof(float) * (size_t)m->n, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "md get");
    }
    m->parent->launches += c->launches;
    c->launches = 0;
    return sync_and_check(c, "md get");
}

nd_status md_energy(MDEngine* m, double* pot, double* kin) {
    Ctx* c = &m->sub;
    nd_status st = md_measure(m, true);
    if (st) return st;
    const int32_t ns = std::max(m->nsys, 1);
    std::vector<double> h(2 * (size_t)ns);
    cudaError_t e = cudaMemcpyAsync(h.data(), m->acc.p, sizeof(double) * h.size(),
                                    cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "md energy");
    m->parent->launches += c->launches;
    c->launches = 0;
    if ((st = sync_and_check(c, "md energy"))) return st;
    double up = 0.0, uk = 0.0;
    for (int32_t k = 0; k < ns; ++k) { up += h[2 * k]; uk += h[2 * k + 1]; }
    if (pot) *pot = up;
    if (kin) *kin = uk;
    return ND_OK;
}

nd_status md_energies(MDEngine* m, double* pot, double* kin) {
    Ctx* c = &m->sub;
    if (m->nsys <= 0) return ND_ERR_ARG;
    nd_status st = md_measure(m, true);
    if (st) return st;
    std::vector<double> h(2 * (size_t)m->nsys);
    cudaError_t e = cudaMemcpyAsync(h.data(), m->acc.p, sizeof(double) * h.size(),
                                    cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "batch energies");
    m->parent->launches += c->launches;
    c->launches = 0;
    if ((st = sync_and_check(c, "batch energies"))) return st;
    for (int32_t k = 0; k < m->nsys; ++k) {
        if (pot) pot[k] = h[2 * k];
        if (kin) kin[k] = h[2 * k + 1];
    }
    return ND_OK;
}

nd_status md_stats(MDEngine* m, int64_t* steps, int64_t* rebuilds, int64_t* list_pairs,
                   int32_t* capacity) {
    if (steps) *steps = m->steps;
    if (rebuilds) *rebuilds = m->rebuilds;
    if (capacity) *capacity = m->lcap;
    if (list_pairs) {
        // sum of ncount (full list: each pair twice)
        std::vector<int32_t> h(m->n);
        cudaError_t e = cudaMemcpyAsync(h.data(), m->ncount.p, sizeof(int32_t) * (size_t)m->n,
                                        cudaMemcpyDeviceToHost, m->sub.stream);
        if (e != cudaSuccess) return cuda_fail(&m->sub, e, "md stats");
        e = cudaStreamSynchronize(m->sub.stream);
        if (e != cudaSuccess) return cuda_fail(&m->sub, e, "md stats");
        int64_t s = 0;
        for (int32_t v : h) s += (v & 0xffff) + (v >> 16);
        *list_pairs = s;
    }
    return ND_OK;
}

// Entries of the current lists as directed pairs of 1-based caller indices
// (each unordered pair once from each side), with the near-segment flag, in
// no particular order.
__global__ void k_md_list_pairs(const int32_t* __restrict__ ncount,
                                const uint16_t* __restrict__ llist,
                                const int32_t* __restrict__ ulist, const int32_t* __restrict__ orig,
                                int32_t n, int32_t apl, int32_t ucap, int32_t lcap,
                                int32_t* __restrict__ pi, int32_t* __restrict__ pj,
                                uint8_t* __restrict__ near, int64_t cap,
                                unsigned long long* cursor) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t b = i / kBlock, t = i - b * kBlock;
    const int32_t c = ncount[i];
    const uint16_t* L = llist + (int64_t)b * lcap * kBlock;
    const int32_t* U = ulist + (int64_t)b * ucap;
    const int32_t tot = list_total(c), nn = list_near(c);
    for (int32_t s = 0; s < tot; ++s) {
        const int32_t li = L[llist_at(list_slot(s, c, lcap), t)];
        const int32_t j = U[li / apl] * apl + li % apl;
        const unsigned long long k = atomicAdd(cursor, 1ull);
        if ((int64_t)k < cap) {
            pi[k] = orig[i] + 1;
            pj[k] = orig[j] + 1;
            near[k] = s < nn ? 1 : 0;
        }
    }
}

nd_status md_list_pairs(MDEngine* m, int32_t* pi, int32_t* pj, uint8_t* near, int64_t cap,
                        int64_t* count) {
    Ctx* c = &m->sub;
    nd_status st = sync_and_check(c, "md list pairs");
    if (st) return st;
    int32_t *dpi = nullptr, *dpj = nullptr;
    uint8_t* dn = nullptr;
    unsigned long long* cur = nullptr;
    const size_t k = (size_t)std::max<int64_t>(cap, 1);
    cudaError_t e = cudaMalloc(&dpi, k * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&dpj, k * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&dn, k);
    if (e == cudaSuccess) e = cudaMalloc(&cur, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemsetAsync(cur, 0, sizeof(unsigned long long), c->stream);
    unsigned long long total = 0;
    if (e == cudaSuccess) {
        k_md_list_pairs<<<(unsigned)cdiv(m->n, 256), 256, 0, c->stream>>>(
            (const int32_t*)m->ncount.p, (const uint16_t*)m->llist.p, (const int32_t*)m->ulist.p,
            m->set[m->cur].orig, m->n, m->apl, m->ucap, m->lcap, dpi, dpj, dn, cap, cur);
        c->launches++;
        e = cudaMemcpyAsync(&total, cur, sizeof(total), cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    const int64_t got = std::min<int64_t>((int64_t)total, cap);
    if (e == cudaSuccess && got > 0 && pi) e = cudaMemcpy(pi, dpi, got * sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && got > 0 && pj) e = cudaMemcpy(pj, dpj, got * sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && got > 0 && near) e = cudaMemcpy(near, dn, got, cudaMemcpyDeviceToHost);
    cudaFree(dpi);
    cudaFree(dpj);
    cudaFree(dn);
    cudaFree(cur);
    if (e != cudaSuccess) return cuda_fail(c, e, "md list pairs");
    m->parent->launches += c->launches;
    c->launches = 0;
    if (count) *count = (int64_t)total;
    return (int64_t)total > cap ? ND_NEED_REALLOC : ND_OK;
}

nd_status md_diagnostics(MDEngine* m, nd_md_diag* out) {
    Ctx* c = &m->sub;
    unsigned long long d[2] = {0, 0};
    unsigned ctl[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    unsigned long long ob[2] = {0, 0};
    cudaError_t e = cudaMemcpyAsync(d, m->diag.p, sizeof(d), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ob, m->obs.p, sizeof(ob), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctl, m->ctl.p, sizeof(ctl), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "md diagnostics");
    *out = nd_md_diag{};
    out->skin_violations = (int64_t)d[0];
    // diag int32 words 2 and 3 hold the largest union and list seen
    out->max_neighbors = (int32_t)(d[1] >> 32);
    out->resorts = ctl[6];
    out->refits = ctl[7];
    out->early_refits = ctl[2];
    out->resort_kernels = m->resort_kernels;
    out->refit_kernels = m->refit_kernels;
    // kernels run inside conditional bodies of graphs: all bodies run, less
    // those the host ran (and counted) itself
    out->body_kernels = (int64_t)ctl[6] * m->resort_kernels +
                        ((int64_t)ctl[7] + ctl[2]) * m->refit_kernels +
                        (int64_t)ob[1] * m->thermo_kernels + (int64_t)ob[0] * m->log_kernels -
                        m->eager_bodies;
    return ND_OK;
}

int64_t md_launches_per_run(MDEngine* m, int64_t steps) {
    const int64_t R = m->p.rebuild_every;
    return (steps / R) * m->graph_main_launches + (steps % R);
}

nd_status md_sync(MDEngine* m) { return sync_and_check(&m->sub, "md sync"); }

// Re-capture the window graphs after a change of the observers.
static nd_status md_recapture(MDEngine* m) {
    if (!m->cap_stream) return ND_OK;
    Ctx* c = &m->sub;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "recapture");
    if (m->graph_main) { cudaGraphExecDestroy(m->graph_main); m->graph_main = nullptr; }
    if (m->graph_first) { cudaGraphExecDestroy(m->graph_first); m->graph_first = nullptr; }
    nd_status st = md_capture_main(m);
    if (st == ND_OK) st = md_capture_first(m);
    return st;
}

nd_status md_set_thermostat(MDEngine* m, double temperature, double gamma, int32_t every) {
    if (every < 0 || !std::isfinite(temperature) || !std::isfinite(gamma)) return ND_ERR_ARG;
    if (every > 0 && m->nsys > 0) {
        m->sub.last_error = "the thermostat applies to single-system engines";
        return ND_ERR_ARG;
    }
    m->thermo_T = temperature;
    m->thermo_gamma = gamma;
    m->thermo_every = every;
    return md_recapture(m);
}

nd_status md_set_log(MDEngine* m, int32_t every, int32_t frames) {
    if (every < 0 || (every > 0 && frames <= 0)) return ND_ERR_ARG;
    Ctx* c = &m->sub;
    if (every > 0) {
        nd_status st = ensure(c, m->logbuf, sizeof(double) * 3 * (size_t)m->n * (size_t)frames);
        if (st) return st;
    }
    m->log_every = every;
    m->log_frames = every > 0 ? frames : 0;
    if (cudaMemsetAsync(m->obs.p, 0, sizeof(unsigned long long), c->stream) != cudaSuccess)
        return cuda_fail(c, cudaGetLastError(), "position log");
    return md_recapture(m);
}

nd_status md_log_count(MDEngine* m, int64_t* count) {
    unsigned long long v = 0;
    Ctx* c = &m->sub;
    cudaError_t e = cudaMemcpyAsync(&v, m->obs.p, sizeof(v), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "position log");
    *count = (int64_t)v;
    return ND_OK;
}

nd_status md_log_read(MDEngine* m, int64_t first, int64_t nframes, double* out) {
    Ctx* c = &m->sub;
    int64_t count = 0;
    nd_status st = md_log_count(m, &count);
    if (st) return st;
    if (m->log_frames <= 0 || first < 0 || nframes < 0 || first + nframes > count ||
        first < count - m->log_frames) {
        c->last_error = "frames outside the position log";
        return ND_ERR_ARG;
    }
    const size_t fb = sizeof(double) * 3 * (size_t)m->n;
    for (int64_t k = 0; k < nframes; ++k) {
        const int64_t slot = (first + k) % m->log_frames;
        cudaError_t e = cudaMemcpyAsync((char*)out + k * fb, (const char*)m->logbuf.p + slot * fb,
                                        fb, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "position log");
    }
    return sync_and_check(c, "position log");
}

const char* md_last_error(MDEngine* m) { return m->sub.last_error.c_str(); }

nd_status forces_pairs(Ctx* c, const nd_md_params* p, int32_t n, const double* x,
                       const double* q, const int32_t* pi, const int32_t* pj, int64_t np,
                       float* f, double* energy) {
    if (!p || !x || !f || n <= 0 || np < 0 || (np > 0 && (!pi || !pj))) return ND_ERR_ARG;
    const size_t nx = 3 * (size_t)n;
    size_t need = nx * sizeof(double) + (q ? n * sizeof(double) : 0) + nx * sizeof(float) +
                  2 * sizeof(int32_t) * (size_t)np + 64;
    nd_status st = ensure(c, c->misc, need);
    if (st) return st;
    char* b = (char*)c->misc.p;
    double* acc = (double*)b;
    double* dx = (double*)(b + 64);
    double* dq = dx + nx;
    float* df = (float*)(dq + (q ? n : 0));
    int32_t* dpi = (int32_t*)(df + nx);
    int32_t* dpj = dpi + np;
    cudaError_t e = cudaMemcpyAsync(dx, x, nx * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && q) e = cudaMemcpyAsync(dq, q, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && np)
        e = cudaMemcpyAsync(dpi, pi, np * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && np)
        e = cudaMemcpyAsync(dpj, pj, np * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "pair forces upload");
    cudaMemsetAsync(df, 0, nx * sizeof(float), c->stream);
    cudaMemsetAsync(acc, 0, sizeof(double), c->stream);
    if (np > 0) {
        int blocks = (int)std::min<int64_t>(cdiv(np, 256), 152 * 16);
        bool coul = q && p->coulomb_k != 0.0;
        k_pair_forces<<<blocks, 256, 0, c->stream>>>(
            dx, coul ? dq : nullptr, dpi, dpj, np, n, (float)(p->cutoff * p->cutoff),
            (float)(p->sigma * p->sigma), (float)(24.0 * p->epsilon), (float)(4.0 * p->epsilon),
            (float)p->coulomb_k, df, acc, c->d_err);
        c->launches++;
    }
    double hacc = 0.0;
    e = cudaMemcpyAsync(f, df, nx * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hacc, acc, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "pair forces download");
    st = sync_and_check(c, "pair forces");
    if (st == ND_OK && energy) *energy = hacc;
    return st;
}

}  // namespace nd
