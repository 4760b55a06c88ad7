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
#include <vector>

#include "nd_internal.cuh"

namespace nd {

constexpr int kBlock = 256;          // atoms per block in the list and step kernels
constexpr int kSizingFcap = 8192;    // BFS frontier entries per buffer in the sizing build
constexpr int kSizingUcap = 8192;    // union capacity of the sizing build

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
};

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
                                  int32_t n, double* q, double* im, int32_t* orig) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    q[i] = q_in ? q_in[i] : 0.0;
    im[i] = m_in ? 1.0 / m_in[i] : 1.0;
    orig[i] = i;
}

__global__ void k_md_pos32(const double* __restrict__ x0, const double* __restrict__ x1,
                           const double* __restrict__ x2, int32_t n, float* __restrict__ xyz) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    xyz[3 * (int64_t)i] = (float)x0[i];
    xyz[3 * (int64_t)i + 1] = (float)x1[i];
    xyz[3 * (int64_t)i + 2] = (float)x2[i];
}

__device__ __forceinline__ int32_t to_fixed(double x, double o, double s, int32_t* err,
                                            int32_t who) {
    double t = fma(x, s, -(o * s));
    if (!(t > -2147483000.0 && t < 2147483000.0)) {
        set_error(err, isfinite(x) ? ND_ERR_RANGE : ND_ERR_NONFINITE, who);
        t = 0.0;
    }
    return __double2int_rn(t);
}

// Gather every per-atom array into the new (sorted) order; write the pair
// records and the Float32 positions of the tree.
__global__ void k_md_reorder(SetPtrs src, SetPtrs dst, const int32_t* __restrict__ perm,
                             const float* __restrict__ xyz32, int32_t n, Frame fr,
                             float4* __restrict__ pos32, int4* __restrict__ rec,
                             int4* __restrict__ recb, int32_t* err) {
    int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int32_t o = perm[k];
    int32_t f[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double xv = src.x[d][o];
        dst.x[d][k] = xv;
        dst.w[d][k] = src.w[d][o];
        f[d] = to_fixed(xv, fr.o[d], fr.s, err, k);
    }
    double qv = src.q[o];
    dst.q[k] = qv;
    dst.im[k] = src.im[o];
    dst.orig[k] = src.orig[o];
    pos32[k] = make_float4(xyz32[3 * (int64_t)o], xyz32[3 * (int64_t)o + 1],
                           xyz32[3 * (int64_t)o + 2], __int_as_float(k));
    rec[k] = make_int4(f[0], f[1], f[2], __float_as_int((float)qv));
    recb[k] = rec[k];
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

// One block per 256 atoms: the boxes of its eight warps (their atoms -/+ hq)
// are tested against the tree breadth-first -- all 256 threads expand the
// current level together, a node's children being (left, skip of left) in the
// rope layout -- and every leaf overlapping any of them joins the union.  The union is sorted (bitonic)
// so list order, and hence force summation order, is deterministic.
// Shared memory: two frontier buffers of fcap entries and the union (upow2).
__global__ void __launch_bounds__(kBlock)
    k_md_block_union(const float4* __restrict__ keys, const float4* __restrict__ pos,
                     int32_t n, int32_t nL, int32_t apl, float hq, int32_t fcap, int32_t ucap,
                     int32_t upow2, int32_t* __restrict__ ulist, int32_t* __restrict__ ucount,
                     uint16_t* __restrict__ llist_leaf, int32_t* __restrict__ lcount_leaf,
                     int32_t lcap_leaf, int32_t* err, int32_t* diag, int32_t sizing) {
    extern __shared__ int32_t smem[];
    int32_t* fr[2] = {smem, smem + fcap};
    int32_t* su = smem + 2 * fcap;
    __shared__ int32_t s_cnt[2];
    __shared__ int32_t s_nu;
    __shared__ float s_wb[kBlock / 32][6];  // per-warp query boxes (min xyz, max xyz)
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t i = (int64_t)blockIdx.x * kBlock + tid;
    float mn[3], mx[3];
    {
        float4 p = pos[i < n ? i : (int64_t)blockIdx.x * kBlock];
        mn[0] = mx[0] = p.x; mn[1] = mx[1] = p.y; mn[2] = mx[2] = p.z;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d)
        for (int s = 16; s > 0; s >>= 1) {
            mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], s));
            mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], s));
        }
    if (lane == 0)
        for (int d = 0; d < 3; ++d) { s_wb[warp][d] = mn[d] - hq; s_wb[warp][3 + d] = mx[d] + hq; }
    if (tid == 0) { s_cnt[0] = 1; s_cnt[1] = 0; s_nu = 0; fr[0][0] = (nL + 1) << 1; }
    __syncthreads();
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
            for (int w = 0; w < kBlock / 32 && !hit; ++w)
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
    const int32_t nu = s_nu;
    if (tid == 0) { atomicMax(&diag[0], nu); atomicAdd(&diag[3], nu); }
    if (nu > ucap) {
        if (tid == 0 && !sizing) set_error(err, ND_ERR_OVERFLOW, (int32_t)blockIdx.x);
        if (tid == 0) ucount[blockIdx.x] = 0;
        for (int32_t k = tid; k < kBlock / apl; k += kBlock) {
            const int64_t leaf = (int64_t)blockIdx.x * (kBlock / apl) + k;
            if (leaf < nL) lcount_leaf[leaf] = 0;
        }
        return;
    }
    // bitonic sort of the union (padded to a power of two)
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
    int32_t* dst = ulist + (int64_t)blockIdx.x * ucap;
    for (int32_t k = tid; k < nu; k += kBlock) dst[k] = su[k];
    if (tid == 0) ucount[blockIdx.x] = nu;
    // Per-leaf candidate lists: for each of its leaves a warp keeps the union
    // positions whose leaf box overlaps that leaf's box (the leaf-leaf test of
    // leafneighbor_traverse, BVHTraverse.jl:1282), ballot-compacted in union
    // order.  A lane loads one union box per chunk and tests it against up to
    // eight own leaves.  The own boxes are widened by a few ulps so no pair is
    // lost to rounding; the atom distance test decides.
    __shared__ float s_own[kBlock / 32][8][6];
    const unsigned below = (1u << lane) - 1u;
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
        int32_t lc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int32_t base = 0; base < nu; base += 32) {
            const int32_t u = base + lane;
            float4 a = make_float4(1.f, 1.f, 1.f, -1.f), b = make_float4(-1.f, -1.f, 0.f, 0.f);
            if (u < nu) {
                const int32_t leaf = su[u];
                a = __ldg(&keys[2 * (int64_t)leaf]);
                b = __ldg(&keys[2 * (int64_t)leaf + 1]);
            }
#pragma unroll
            for (int kl = 0; kl < 8; ++kl) {
                if (kl >= nown) break;
                const float* o = s_own[warp][kl];
                const bool hit = (u < nu) && box_overlap(o[0], o[1], o[2], o[3], o[4], o[5], a, b);
                const unsigned m = __ballot_sync(0xffffffffu, hit);
                if (hit) {
                    const int32_t pos = lc[kl] + __popc(m & below);
                    if (pos < lcap_leaf) llist_leaf[(first_own + k0 + kl) * lcap_leaf + pos] = (uint16_t)u;
                }
                lc[kl] += __popc(m);
            }
        }
        if (lane < nown) {
            int32_t mine = 0;
#pragma unroll
            for (int kl = 0; kl < 8; ++kl)
                if (kl == lane) mine = lc[kl];
            const int64_t own = first_own + k0 + lane;
            if (own < nL) {
                lcount_leaf[own] = min(mine, lcap_leaf);
                atomicMax(&diag[2], mine);
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
// as uint16.  pos.w holds the atom's sorted index (excludes the atom itself).
template <int APL>
__global__ void __launch_bounds__(kBlock)
    k_md_block_lists(const float4* __restrict__ pos, int32_t n, float rl2, int32_t ucap,
                     int32_t smpos, const int32_t* __restrict__ ulist,
                     const int32_t* __restrict__ ucount, const uint16_t* __restrict__ llist_leaf,
                     const int32_t* __restrict__ lcount_leaf, int32_t lcap_leaf, int32_t lcap,
                     uint16_t* __restrict__ llist, int32_t* __restrict__ ncount, int32_t* err,
                     int32_t* diag, int32_t sizing) {
    extern __shared__ float4 spos[];
    const int tid = threadIdx.x;
    const int32_t* __restrict__ U = ulist + (int64_t)blockIdx.x * ucap;
    {
        const int32_t nu = min(__ldg(&ucount[blockIdx.x]), ucap);
        const int32_t m = min(nu * APL, smpos);
        for (int32_t k = tid; k < m; k += kBlock)
            spos[k] = __ldg(&pos[(int64_t)__ldg(&U[k / APL]) * APL + (k % APL)]);
    }
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * kBlock + tid;
    const bool valid = i < n;
    const int64_t own = (valid ? i : (int64_t)blockIdx.x * kBlock) / APL;
    const float4 p = __ldg(&pos[valid ? i : (int64_t)blockIdx.x * kBlock]);
    const int32_t nc = valid ? min(__ldg(&lcount_leaf[own]), lcap_leaf) : 0;
    const uint16_t* __restrict__ C = llist_leaf + own * lcap_leaf;
    uint16_t* __restrict__ L = llist + (int64_t)blockIdx.x * lcap * kBlock + tid;
    const int32_t self = (int32_t)i;
    int32_t cnt = 0;
    for (int32_t k = 0; k < nc; ++k) {
        const int32_t u = __ldg(&C[k]);
        float4 q[APL];
        if ((u + 1) * APL <= smpos) {
#pragma unroll
            for (int e = 0; e < APL; ++e) q[e] = spos[u * APL + e];
        } else {
            const int64_t base = (int64_t)__ldg(&U[u]) * APL;
#pragma unroll
            for (int e = 0; e < APL; ++e) q[e] = __ldg(&pos[base + e]);
        }
#pragma unroll
        for (int e = 0; e < APL; ++e) {
            const bool hit = dist2_ref(p.x, p.y, p.z, q[e].x, q[e].y, q[e].z) < rl2 &&
                             __float_as_int(q[e].w) != self;
            if (hit) {
                if (cnt < lcap) L[(int64_t)cnt * kBlock] = (uint16_t)(u * APL + e);
                ++cnt;
            }
        }
    }
    if (!valid) return;
    ncount[i] = min(cnt, lcap);
    if (cnt > lcap && !sizing) set_error(err, ND_ERR_OVERFLOW, (int32_t)i);
    atomicMax(&diag[1], cnt);
}

// Refit: positions changed, order and tree topology kept.  Float32 positions
// and pair records (and the build records of the skin check) from the FP64
// state in its current order.
__global__ void k_md_refit_pos(SetPtrs st, int32_t n, Frame fr, float4* __restrict__ pos32,
                               int4* __restrict__ rec, int4* __restrict__ recb, int32_t* err) {
    int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int32_t f[3];
    float xf[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double xv = st.x[d][k];
        xf[d] = (float)xv;
        f[d] = to_fixed(xv, fr.o[d], fr.s, err, k);
    }
    pos32[k] = make_float4(xf[0], xf[1], xf[2], __int_as_float(k));
    int4 r = make_int4(f[0], f[1], f[2], __float_as_int((float)st.q[k]));
    rec[k] = r;
    recb[k] = r;
}

// ------------------------------------------------------------- step kernel

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
};

// Pair (i, j) from fixed-point records: the integer difference is exact, its
// conversion to float rounds once, so r_ij keeps full single precision at any
// box size inside the frame.  Constants are pre-scaled, so the force comes out
// in physical units per fixed-point unit of displacement.
template <bool COUL, bool ENERGY>
__device__ __forceinline__ void accum_pair(const int4& ri, const int4& rj, const StepArgs& a,
                                          float& fx, float& fy, float& fz, float& ue) {
    const float dx = (float)(ri.x - rj.x);
    const float dy = (float)(ri.y - rj.y);
    const float dz = (float)(ri.z - rj.z);
    const float r2 = dx * dx + dy * dy + dz * dz;
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
        float u = 0.f;
        if (ENERGY) u = a.eps4 * s6 * (s6 - 1.0f);
        if (COUL) {
            const float qq = __int_as_float(ri.w) * __int_as_float(rj.w);
            fmag += a.kcu * qq * inv_r * inv_r2;
            if (ENERGY) u += a.kceu * qq * inv_r;
        }
        fx += fmag * dx;
        fy += fmag * dy;
        fz += fmag * dz;
        if (ENERGY) ue += u;
    }
}

// One block per 256 atoms.  MODE 0: step (force, pending half kick, kick,
// drift, reflect, next record).  MODE 1: measure (force, integer-step velocity
// and energies; state untouched).
template <bool COUL, bool MASS, bool FIRST, int MODE>
__global__ void __launch_bounds__(kBlock, 4) k_md_step(StepArgs a) {
    extern __shared__ int4 srec[];
    const int tid = threadIdx.x;
    int64_t i = (int64_t)blockIdx.x * kBlock + tid;
    const bool valid = i < a.n;
    const int32_t* __restrict__ U = a.ulist + (int64_t)blockIdx.x * a.ucap;
    // stage the block's union: record of atom (leaf * apl + e) at u * apl + e,
    // up to the shared-memory capacity; larger unions read the rest from L2
    {
        const int32_t nu = min(__ldg(&a.ucount[blockIdx.x]), a.ucap);
        const int32_t m = min(nu * a.apl, a.smrec);
        for (int32_t k = tid; k < m; k += kBlock) {
            const int32_t u = k / a.apl, e = k - u * a.apl;
            srec[k] = __ldg(&a.rec_in[(int64_t)__ldg(&U[u]) * a.apl + e]);
        }
    }
    __syncthreads();
    if (MODE == 0 && !valid) return;
    if (!valid) i = a.n - 1;  // measure: idle lanes join the warp reduction with zeros
    const int4 ri = __ldg(&a.rec_in[i]);
    const int32_t cnt = valid ? __ldg(&a.ncount[i]) : 0;
    const uint16_t* __restrict__ L = a.llist + (int64_t)blockIdx.x * a.lcap * kBlock + tid;
    auto fetch = [&](int32_t li) -> int4 {
        if (li < a.smrec) return srec[li];
        const int32_t u = li / a.apl, e = li - u * a.apl;
        return __ldg(&a.rec_in[(int64_t)__ldg(&U[u]) * a.apl + e]);
    };
    float fx = 0.f, fy = 0.f, fz = 0.f, ue = 0.f;
    // groups of four neighbours; the next group's indices are loaded while the
    // current group is computed
    int32_t s = 0;
    int32_t li[4];
    if (cnt >= 4) {
#pragma unroll
        for (int k = 0; k < 4; ++k) li[k] = L[(int64_t)k * kBlock];
    }
    for (; s + 4 <= cnt; s += 4) {
        int4 rj[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) rj[k] = fetch(li[k]);
        if (s + 8 <= cnt) {
#pragma unroll
            for (int k = 0; k < 4; ++k) li[k] = L[(int64_t)(s + 4 + k) * kBlock];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) accum_pair<COUL, MODE == 1>(ri, rj[k], a, fx, fy, fz, ue);
    }
    for (; s < cnt; ++s) accum_pair<COUL, MODE == 1>(ri, fetch(L[(int64_t)s * kBlock]), a, fx, fy, fz, ue);
    if (valid) a.f_out[i] = make_float4(fx, fy, fz, 0.f);
    const double imv = MASS ? a.im[i] : 1.0;
    const float fv[3] = {fx, fy, fz};
    if constexpr (MODE == 1) {
        double ke = 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double kick = (double)(a.hdt * fv[d]) * imv;
            double v = FIRST ? a.w[d][i] : a.w[d][i] + kick;
            if (valid) a.v_out[d][i] = v;
            ke += v * v;
        }
        double mass = MASS ? 1.0 / imv : 1.0;
        double pe = valid ? 0.5 * (double)ue : 0.0;
        ke = valid ? ke * 0.5 * mass : 0.0;
        for (int sh = 16; sh > 0; sh >>= 1) {
            pe += __shfl_xor_sync(0xffffffffu, pe, sh);
            ke += __shfl_xor_sync(0xffffffffu, ke, sh);
        }
        if ((tid & 31) == 0) {
            atomicAdd(&a.acc[0], pe);
            atomicAdd(&a.acc[1], ke);
        }
        return;
    } else {
        // v_{n+1/2} = v_{n-1/2} + dt F/m (the pending half kick and this step's
        // half kick in one add), x += dt v, walls, next record.
        const float kdt = FIRST ? a.hdt : 2.0f * a.hdt;
        int32_t xi[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double v = a.w[d][i] + (double)(kdt * fv[d]) * imv;
            double x = fma(a.dt, v, a.x[d][i]);
            int32_t q = __double2int_rn(fma(x, a.fr.s, -a.os[d]));
            // integer pre-check; the exact FP64 test of boundary_reflect! runs
            // only for atoms within a grid step of a wall
            if (q <= a.lo_fp[d] + 1 || q >= a.hi_fp[d] - 1) {
                if (a.lo[d] > x) { v = -v; x = a.lo[d]; }
                if (a.hi[d] < x) { v = -v; x = a.hi[d]; }
                q = __double2int_rn(fma(x, a.fr.s, -a.os[d]));
                if (!(x == x)) set_error(a.err, ND_ERR_NONFINITE, (int32_t)i);
            }
            a.x[d][i] = x;
            a.w[d][i] = v;
            xi[d] = q;
        }
        a.rec_out[i] = make_int4(xi[0], xi[1], xi[2], ri.w);
        // A list built at r_c + skin stays valid while no atom moved more than
        // skin/2 since the build; count the atom-steps that broke that bound.
        const int4 rb = __ldg(&a.rec_build[i]);
        const float ex = (float)(xi[0] - rb.x), ey = (float)(xi[1] - rb.y),
                    ez = (float)(xi[2] - rb.z);
        if (ex * ex + ey * ey + ez * ez > a.half_skin2u) atomicAdd(a.diag, 1ull);
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
    DevBuf set_buf[2], rec_buf[2], recb, xyz32, pos32, keys, store, ulist, ucount, llist_leaf,
        lcount_leaf, llist, ncount, f, vtmp, acc, aos, diag;
    SetPtrs set[2];
    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [refit][set]
    int32_t resort_every = 5;  // re-sort (new order + topology) every k-th rebuild, refit between
    int64_t graph_launches[2] = {0, 0};  // kernels per captured window [refit]
    size_t step_smem = 0, union_smem = 0, lists_smem = 0;
};

static nd_status md_alloc(MDEngine* m) {
    Ctx* c = &m->sub;
    const size_t n = (size_t)m->n;
    nd_status st;
    for (int s = 0; s < 2; ++s) {
        // x[3], w[3], q, im (8 doubles) + orig (int32)
        if ((st = ensure(c, m->set_buf[s], n * (8 * sizeof(double) + sizeof(int32_t)) + 256))) return st;
        double* b = (double*)m->set_buf[s].p;
        for (int d = 0; d < 3; ++d) { m->set[s].x[d] = b + d * n; m->set[s].w[d] = b + (3 + d) * n; }
        m->set[s].q = b + 6 * n;
        m->set[s].im = b + 7 * n;
        m->set[s].orig = (int32_t*)(b + 8 * n);
        if ((st = ensure(c, m->rec_buf[s], n * sizeof(int4)))) return st;
    }
    if ((st = ensure(c, m->recb, n * sizeof(int4)))) return st;
    if ((st = ensure(c, m->lcount_leaf, sizeof(int32_t) * (size_t)m->nL))) return st;
    if ((st = ensure(c, m->xyz32, 3 * n * sizeof(float)))) return st;
    if ((st = ensure(c, m->pos32, n * sizeof(float4)))) return st;
    if ((st = ensure(c, m->keys, 32 * (size_t)(2 * m->nL)))) return st;
    if ((st = ensure(c, m->store, sizeof(int32_t) * (size_t)m->nL))) return st;
    if ((st = ensure(c, m->ucount, sizeof(int32_t) * (size_t)m->nblocks))) return st;
    if ((st = ensure(c, m->ncount, sizeof(int32_t) * n))) return st;
    if ((st = ensure(c, m->f, sizeof(float4) * n))) return st;
    if ((st = ensure(c, m->vtmp, 3 * sizeof(double) * n))) return st;
    if ((st = ensure(c, m->acc, 64))) return st;
    if ((st = ensure(c, m->diag, 64))) return st;
    if (cudaMemsetAsync(m->diag.p, 0, 64, c->stream) != cudaSuccess) return ND_ERR_CUDA;
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
    if ((st = ensure(c, m->ulist, sizeof(int32_t) * (size_t)ucap * m->nblocks))) return st;
    if (lcap > 0 &&
        (st = ensure(c, m->llist, sizeof(uint16_t) * (size_t)lcap * kBlock * m->nblocks)))
        return st;
    if (lcap_leaf > 0 &&
        (st = ensure(c, m->llist_leaf, sizeof(uint16_t) * (size_t)lcap_leaf * m->nL)))
        return st;
    m->union_smem = sizeof(int32_t) * (2 * (size_t)fcap + p2);
    m->step_smem = sizeof(int4) * (size_t)m->ucap_sm * m->apl;
    m->lists_smem = sizeof(float4) * (size_t)m->ucap_sm * m->apl;
    int maxsm = 0;
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
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
#define ND_SMEM(C, M, F, MODE) \
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_md_step<C, M, F, MODE>, maxsm);
    ND_SMEM(true, true, true, 0) ND_SMEM(true, true, false, 0) ND_SMEM(true, false, true, 0)
    ND_SMEM(true, false, false, 0) ND_SMEM(false, true, true, 0)
    ND_SMEM(false, true, false, 0) ND_SMEM(false, false, true, 0)
    ND_SMEM(false, false, false, 0) ND_SMEM(true, true, true, 1)
    ND_SMEM(true, true, false, 1) ND_SMEM(true, false, true, 1)
    ND_SMEM(true, false, false, 1) ND_SMEM(false, true, true, 1)
    ND_SMEM(false, true, false, 1) ND_SMEM(false, false, true, 1)
    ND_SMEM(false, false, false, 1)
#undef ND_SMEM
    if (e != cudaSuccess) return cuda_fail(c, e, "shared memory opt-in");
    return ND_OK;
}

static StepArgs md_step_args(MDEngine* m, int rec_in) {
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
    const float hs = (float)(0.5 * p.skin * S);
    a.half_skin2u = hs * hs;
    for (int d = 0; d < 3; ++d) {
        a.os[d] = m->fr.o[d] * S;
        a.lo_fp[d] = (int32_t)std::floor((p.box_lo[d] - m->fr.o[d]) * S);
        a.hi_fp[d] = (int32_t)std::ceil((p.box_hi[d] - m->fr.o[d]) * S);
    }
    a.rc2u = (float)(p.cutoff * p.cutoff * S * S);
    a.sig2u = (float)(p.sigma * p.sigma * S * S);
    a.eps24u = (float)(24.0 * p.epsilon * S);
    a.eps4 = (float)(4.0 * p.epsilon);
    a.kcu = (float)(p.coulomb_k * S * S);
    a.kceu = (float)(p.coulomb_k * S);
    a.hdt = (float)(0.5 * p.dt);
    a.dt = p.dt;
    a.fr = m->fr;
    return a;
}

template <int MODE>
static void launch_step(MDEngine* m, const StepArgs& a, bool first) {
    Ctx* c = &m->sub;
    const unsigned grid = (unsigned)m->nblocks;
    const size_t sm = m->step_smem;
    const bool coul = m->has_q && m->p.coulomb_k != 0.0;
    const bool mass = m->has_m;
#define ND_STEP(C, M, F) k_md_step<C, M, F, MODE><<<grid, kBlock, sm, c->stream>>>(a)
    if (coul) {
        if (mass) { if (first) ND_STEP(true, true, true); else ND_STEP(true, true, false); }
        else { if (first) ND_STEP(true, false, true); else ND_STEP(true, false, false); }
    } else {
        if (mass) { if (first) ND_STEP(false, true, true); else ND_STEP(false, true, false); }
        else { if (first) ND_STEP(false, false, true); else ND_STEP(false, false, false); }
    }
#undef ND_STEP
    c->launches++;
}

// Rebuild: Float32 positions -> codes -> sort -> reorder state -> leaf boxes ->
// build -> block unions -> per-atom lists; switches the current state set.
// A refit keeps the order and the sorted codes (so the build reproduces the
// topology) and only refreshes positions, boxes, unions and lists.
static nd_status md_rebuild(MDEngine* m, bool sizing = false, bool refit = false) {
    Ctx* c = &m->sub;
    const int32_t n = m->n;
    const unsigned g = (unsigned)cdiv(n, 256);
    int32_t* codes = (int32_t*)c->codes.p;
    int32_t* perm = (int32_t*)c->perm.p;
    nd_status st;
    if (refit) {
        k_md_refit_pos<<<g, 256, 0, c->stream>>>(m->set[m->cur], n, m->fr, (float4*)m->pos32.p,
                                                  (int4*)m->rec_buf[0].p, (int4*)m->recb.p,
                                                  c->d_err);
        c->launches++;
    } else {
        SetPtrs& s = m->set[m->cur];
        SetPtrs& t = m->set[m->cur ^ 1];
        k_md_pos32<<<g, 256, 0, c->stream>>>(s.x[0], s.x[1], s.x[2], n, (float*)m->xyz32.p);
        c->launches++;
        if ((st = morton_codes(c, (const float*)m->xyz32.p, n, m->p.order, codes, perm))) return st;
        if ((st = radix_sort_pairs(c, (uint32_t*)codes, perm, n, 30))) return st;
        k_md_reorder<<<g, 256, 0, c->stream>>>(s, t, perm, (const float*)m->xyz32.p, n, m->fr,
                                               (float4*)m->pos32.p, (int4*)m->rec_buf[0].p,
                                               (int4*)m->recb.p, c->d_err);
        c->launches++;
    }
    float4* keys = (float4*)m->keys.p;
    const float rl = (float)(m->p.cutoff + m->p.skin);
    k_md_leaf_boxes<<<(unsigned)cdiv(m->nL, 128), 128, 0, c->stream>>>(
        (const float4*)m->pos32.p, m->nL, m->apl, rl / 2.0f, keys);
    c->launches++;
    if ((st = build_internal_nodes(c, keys, (int32_t*)m->store.p, codes, m->nL, m->apl))) return st;
    // query boxes slightly above r_list/2 so the box tests never drop a pair;
    // the distance test alone decides membership
    const float hq = (rl / 2.0f) * 1.0001f + 1e-6f;
    k_md_block_union<<<(unsigned)m->nblocks, kBlock, m->union_smem, c->stream>>>(
        keys, (const float4*)m->pos32.p, n, m->nL, m->apl, hq, m->fcap, m->ucap, m->upow2,
        (int32_t*)m->ulist.p, (int32_t*)m->ucount.p, (uint16_t*)m->llist_leaf.p,
        (int32_t*)m->lcount_leaf.p, m->lcap_leaf, c->d_err, (int32_t*)m->diag.p + 2,
        sizing ? 1 : 0);
#define ND_LISTS(A)                                                                             \
    k_md_block_lists<A><<<(unsigned)m->nblocks, kBlock, m->lists_smem, c->stream>>>(            \
        (const float4*)m->pos32.p, n, rl * rl, m->ucap, m->ucap_sm * m->apl,                    \
        (const int32_t*)m->ulist.p, (const int32_t*)m->ucount.p,                                \
        (const uint16_t*)m->llist_leaf.p, (const int32_t*)m->lcount_leaf.p, m->lcap_leaf,       \
        m->lcap, (uint16_t*)m->llist.p, (int32_t*)m->ncount.p, c->d_err,                        \
        (int32_t*)m->diag.p + 2, sizing ? 1 : 0)
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
    if (!refit) m->cur ^= 1;
    m->rc = 0;
    return check_launch(c, "md rebuild");
}

// Enqueue `k` steps inside the current window (no rebuild).
static void md_steps(MDEngine* m, int32_t k) {
    for (int32_t s = 0; s < k; ++s) {
        StepArgs a = md_step_args(m, m->rc);
        launch_step<0>(m, a, m->first);
        m->first = false;
        m->rc ^= 1;
    }
}

static nd_status md_capture_window(MDEngine* m, int which, int refit) {
    // Captures (re-sort or refit) rebuild + R steps starting from state set `which`.
    Ctx* c = &m->sub;
    int save_cur = m->cur, save_rc = m->rc;
    bool save_first = m->first;
    int64_t save_launch = c->launches;
    m->cur = which;
    m->first = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(c, e, "begin capture");
    nd_status st = md_rebuild(m, false, refit != 0);
    if (st == ND_OK) md_steps(m, m->p.rebuild_every);
    e = cudaStreamEndCapture(c->stream, &g);
    if (st) { if (g) cudaGraphDestroy(g); return st; }
    if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
    e = cudaGraphInstantiate(&m->graph[refit][which], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "graph instantiate");
    m->graph_launches[refit] = c->launches - save_launch;
    c->launches = save_launch;
    m->cur = save_cur;
    m->rc = save_rc;
    m->first = save_first;
    return ND_OK;
}

// Sizing build pass: diag int32 words 2..6 collect the largest union, the
// largest per-atom list, the largest per-leaf candidate list, the sum of
// union sizes and the largest BFS frontier.
static nd_status md_sizing_pass(MDEngine* m, int32_t h[5]) {
    Ctx* c = &m->sub;
    cudaMemsetAsync((int32_t*)m->diag.p + 2, 0, 5 * sizeof(int32_t), c->stream);
    nd_status st = md_rebuild(m, true);
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
    const int32_t ucap_sm = round_up(mean_u * 1.2 + 16, 16);
    if ((st = md_alloc_lists(m, fcap, ucap, lcap_leaf, 0, ucap_sm))) return st;
    if ((st = md_sizing_pass(m, h))) return st;
    const int32_t max_n = h[1];
    int32_t lcap = m->p.max_neighbors > 0 ? m->p.max_neighbors : round_up(max_n * 1.35 + 16, 8);
    if ((st = md_alloc_lists(m, fcap, ucap, lcap_leaf, lcap, ucap_sm))) return st;
    if ((st = md_rebuild(m))) return st;
    m->in_window = 0;
    m->rebuild_due = false;
    m->rebuilds = 1;
    return sync_and_check(c, "md first build");
}

nd_status md_destroy(MDEngine* m);

// Copy x, v (N x 3), q, m (N) from host or device memory into state set 0 in
// the caller's order and reset the step bookkeeping.
static nd_status md_upload(MDEngine* m, const double* xd, const double* vd, const double* qd,
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
    k_md_init_scalars<<<g, 256, 0, c->stream>>>(qd ? aq : nullptr, md_ ? am : nullptr, n, s.q, s.im,
                                                s.orig);
    c->launches += 3;
    if (cudaMemsetAsync(m->diag.p, 0, 64, c->stream) != cudaSuccess) return ND_ERR_CUDA;
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
    if ((st = md_rebuild(m))) return st;
    m->rebuilds = 1;
    return sync_and_check(&m->sub, "md reset");
}

bool md_compatible(MDEngine* m, const nd_md_params* p, int32_t n, bool has_q, bool has_m) {
    return m && m->n == n && m->has_q == has_q && m->has_m == has_m &&
           memcmp(&m->p, p, sizeof(nd_md_params)) == 0;
}

// Fixed-point frame from the walls: a margin of 1/16 of the largest extent on
// every side, scale = the largest power of two that keeps the frame in int32.
static nd_status md_frame(MDEngine* m) {
    double ext = 0.0;
    for (int d = 0; d < 3; ++d) ext = std::max(ext, m->p.box_hi[d] - m->p.box_lo[d]);
    if (!(ext > 0.0) || !std::isfinite(ext)) return ND_ERR_ARG;
    const double margin = ext / 16.0;
    for (int d = 0; d < 3; ++d) m->fr.o[d] = m->p.box_lo[d] - margin;
    const double range = ext + 2.0 * margin;
    int k = (int)std::floor(std::log2(2147480000.0 / range));
    m->fr.s = std::ldexp(1.0, k);
    return ND_OK;
}

static nd_status md_create_common(Ctx* parent, const nd_md_params* p, int32_t n,
                                  const double* xd, const double* vd, const double* qd,
                                  const double* md_, bool host, bool capture, MDEngine** out) {
    if (!parent || !p || !out || !xd || !vd || n <= 0) return ND_ERR_ARG;
    if (p->atomsperleaf <= 0 || n % p->atomsperleaf || n / p->atomsperleaf < 2) return ND_ERR_SPEC;
    if (32 % p->atomsperleaf != 0) return ND_ERR_SPEC;  // a warp holds whole leaves
    if (p->rebuild_every <= 0 || !(p->cutoff > 0) || !(p->skin >= 0) || !(p->dt > 0))
        return ND_ERR_ARG;
    MDEngine* m = new MDEngine();
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
    nd_status st = md_frame(m);
    if (st == ND_OK) st = md_alloc(m);
    if (st) { parent->last_error = m->sub.last_error; md_destroy(m); return st; }
    Ctx* c = &m->sub;
    if ((st = md_upload(m, xd, vd, qd, md_, host))) { parent->last_error = c->last_error; md_destroy(m); return st; }
    m->cur = 0;
    m->first = true;
    if ((st = md_size_lists(m))) { parent->last_error = c->last_error; md_destroy(m); return st; }
    for (int w = 0; capture && w < 4; ++w)
        if ((st = md_capture_window(m, w & 1, w >> 1))) { parent->last_error = c->last_error; md_destroy(m); return st; }
    parent->launches += c->launches;
    c->launches = 0;
    *out = m;
    return ND_OK;
}

nd_status md_create(Ctx* parent, const nd_md_params* p, int32_t n, const double* x,
                    const double* v, const double* q, const double* mass, bool host,
                    bool capture, MDEngine** out) {
    return md_create_common(parent, p, n, x, v, q, mass, host, capture, out);
}

nd_status md_destroy(MDEngine* m) {
    if (!m) return ND_OK;
    for (int r = 0; r < 2; ++r)
        for (int w = 0; w < 2; ++w)
            if (m->graph[r][w]) cudaGraphExecDestroy(m->graph[r][w]);
    DevBuf* bufs[] = {&m->set_buf[0], &m->set_buf[1], &m->rec_buf[0], &m->rec_buf[1], &m->recb,
                      &m->xyz32, &m->pos32, &m->keys, &m->store, &m->ulist, &m->ucount,
                      &m->llist_leaf, &m->lcount_leaf, &m->llist,
                      &m->ncount, &m->f, &m->vtmp, &m->acc, &m->aos, &m->diag, &m->sub.codes,
                      &m->sub.codes_alt, &m->sub.perm, &m->sub.perm_alt, &m->sub.hist,
                      &m->sub.misc};
    if (m->sub.stream) cudaStreamSynchronize(m->sub.stream);
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    delete m;
    return ND_OK;
}

// Advance `steps` steps: whole windows replay the captured graph of the
// current state set (rebuild + R steps); partial windows are enqueued eagerly.
nd_status md_run(MDEngine* m, int64_t steps) {
    Ctx* c = &m->sub;
    const int32_t R = m->p.rebuild_every;
    nd_status st;
    while (steps > 0) {
        if (m->rebuild_due) {
            // every resort_every-th rebuild re-sorts; the others refit
            const int refit = (m->rebuilds % m->resort_every) != 0 ? 1 : 0;
            if (steps >= R && !m->first && m->graph[refit][m->cur]) {
                cudaError_t e = cudaGraphLaunch(m->graph[refit][m->cur], c->stream);
                if (e != cudaSuccess) return cuda_fail(c, e, "graph launch");
                c->launches += m->graph_launches[refit];
                if (!refit) m->cur ^= 1;
                m->rc = R & 1;
                m->rebuilds++;
                m->steps += R;
                steps -= R;
                continue;
            }
            if ((st = md_rebuild(m, false, refit != 0))) return st;
            m->rebuilds++;
            m->rebuild_due = false;
            m->in_window = 0;
        }
        int32_t k = (int32_t)std::min<int64_t>(steps, R - m->in_window);
        md_steps(m, k);
        m->in_window += k;
        if (m->in_window == R) { m->in_window = 0; m->rebuild_due = true; }
        m->steps += k;
        steps -= k;
    }
    m->parent->launches += c->launches;
    c->launches = 0;
    return check_launch(c, "md run");
}

nd_status md_measure(MDEngine* m) {
    Ctx* c = &m->sub;
    cudaMemsetAsync(m->acc.p, 0, 2 * sizeof(double), c->stream);
    StepArgs a = md_step_args(m, m->rc);
    launch_step<1>(m, a, m->first);
    return check_launch(c, "md measure");
}

nd_status md_get(MDEngine* m, double* x, double* v, float* f, bool host) {
    Ctx* c = &m->sub;
    nd_status st = md_measure(m);
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
    nd_status st = md_measure(m);
    if (st) return st;
    double h[2];
    cudaError_t e = cudaMemcpyAsync(h, m->acc.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "md energy");
    m->parent->launches += c->launches;
    c->launches = 0;
    if ((st = sync_and_check(c, "md energy"))) return st;
    if (pot) *pot = h[0];
    if (kin) *kin = h[1];
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
        for (int32_t v : h) s += v;
        *list_pairs = s;
    }
    return ND_OK;
}

nd_status md_diagnostics(MDEngine* m, int64_t* skin_violations, int32_t* max_neighbors) {
    Ctx* c = &m->sub;
    unsigned long long d[2] = {0, 0};
    cudaError_t e = cudaMemcpyAsync(d, m->diag.p, sizeof(d), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "md diagnostics");
    if (skin_violations) *skin_violations = (int64_t)d[0];
    // diag int32 words 2 and 3 hold the largest union and list seen
    if (max_neighbors) *max_neighbors = (int32_t)(d[1] >> 32);
    return ND_OK;
}

int64_t md_launches_per_run(MDEngine* m, int64_t steps) {
    const int64_t R = m->p.rebuild_every;
    const int64_t w = steps / R, full = (w + m->resort_every - 1) / m->resort_every;
    return full * m->graph_launches[0] + (w - full) * m->graph_launches[1] + (steps % R);
}

nd_status md_sync(MDEngine* m) { return sync_and_check(&m->sub, "md sync"); }

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
