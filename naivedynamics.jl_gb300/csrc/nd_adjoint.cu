// nd_adjoint.cu -- the differentiable form of the hot path: a kick-drift-kick
// trajectory of the MD engine (src/Simulator.jl:154-256 with the intended
// physics of src/Forces.jl and the boundary_reflect! walls of
// src/Simulator.jl:81-111), a Gaussian-smoothed pair-distance histogram of its
// final positions, the squared deviation of that histogram from a target, and
// the hand-written adjoint of all of it: dL/dx0, dL/dv0, dL/dsigma, dL/deps.
// The reference has no derivative code (its differentiation route would be
// ForwardDiff over the CPU path); nothing here has a counterpart in it.
//
// Discrete program (the engine's step kernel, per atom and axis):
//   u_{t+1} = u_t + c_t dt F(x_t)/m      (c_0 = 1/2, c_t = 1 after: the merged kicks)
//   x_{t+1} = x_t + dt u_{t+1};  a coordinate past a wall is clamped to it and
//   its velocity flipped
// Reverse step t (K-1 .. 0), with lx, lu the adjoints of (x_{t+1}, u_{t+1}) and
// M the clamp mask of step t (x_{t+1} equal to a wall):
//   a  = (1 - M) lx                      adjoint of the drifted position
//   g  = (1 - 2M) lu + dt a              adjoint of the kicked velocity
//   lx <- a + c_t dt/m H(x_t) g,  lu <- g,  dL/dtheta += c_t dt/m g . dF/dtheta
// H = dF/dx is symmetric; per atom (H g)_i = sum_j K_ij (g_i - g_j) with
// K = g(r) I + 2 g'(r^2) r r^T for the pair force F_ij = g(r) r_ij, so each
// reverse step is ONE gather kernel over the same neighbour lists as the
// forward step, no atomics.
//
// Memory (sorted order of the engine):
//   ckpt[S]   engine state (x, u, q, 1/m, original index) at every checkpoint
//   perm[S]   the re-sort permutation taken at each checkpoint
//   traj[C]   x_t of the segment being reversed (FP64)
//   abar, gd  FP64 adjoints (3 x N each), g4[2] Float32 copies of gd for the
//             neighbour gather (ping-ponged)
//   hatom     per-atom histogram rows (bins x N Float32) -> h (FP64)
// A segment of C steps is recomputed from its checkpoint before it is
// reversed; the atoms are re-sorted at every checkpoint (the permutation is
// undone on the adjoints when the reverse pass crosses it).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "nd_md_engine.cuh"

namespace nd {

constexpr int kHistChunk = 16;  // histogram bins a thread accumulates per pass
constexpr int kAdjTPA = 4;      // threads per atom in the reverse step

struct AdjArgs {
    int32_t n, apl, ucap, smrec;
    const int32_t* __restrict__ ulist;
    const int32_t* __restrict__ ucount;
    const uint16_t* __restrict__ llist;
    const int32_t* __restrict__ ncount;
    int32_t lcap;
    const double* xt[3];  // positions of the step (sorted order; the wall masks)
    const int4* __restrict__ recs;  // their fixed-point records (x, y, z, charge bits)
    const double* __restrict__ im;
    const float4* __restrict__ g4_in;
    float4* __restrict__ g4_out;
    double* abar[3];
    double* gd[3];
    double* lx0[3];  // last reverse step: dL/dx0, dL/dv0 (sorted order)
    double* lv0[3];
    double* __restrict__ gpart;  // per block: [0] dL/dsigma, [1] dL/deps partial sums
    float invS;
    double lo[3], hi[3];
    float rc2, sig2, eps24, kc;
    double sfac;  // 24 eps / sigma (dF/dsigma factor)
    double ckdt;  // c_t dt
    double dt;
    int32_t last;
    // histogram / loss
    int32_t bins;
    float rmax2, bw, inv2w2, invw2, rsw, inv_span;
    float* __restrict__ hatom;      // bins x n
    const float* __restrict__ cb;   // bins: 2 (h_b - target_b) / N
    int32_t* err;
};

// Atom index (sorted) of union entry li of the block's union U.
__device__ __forceinline__ int64_t adj_atom(const int32_t* __restrict__ U, int32_t li, int32_t apl) {
    const int32_t u = li / apl, e = li - u * apl;
    return (int64_t)__ldg(&U[u]) * apl + e;
}

// Pair kernel of the reverse step in physical units (S is a power of two, so
// scaling the exact integer difference by 1/S rounds only once).
template <bool COUL>
__device__ __forceinline__ void hvp_pair(const AdjArgs& a, const int4& ri, const float4& gi,
                                         const int4& rj, const float4& gj, float3& hv,
                                         float& eacc, float& sacc) {
    const float dx = (float)idiff(ri.x, rj.x) * a.invS;
    const float dy = (float)idiff(ri.y, rj.y) * a.invS;
    const float dz = (float)idiff(ri.z, rj.z) * a.invS;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (!(r2 < a.rc2)) return;
    const float inv_r2 = 1.0f / r2;
    const float s2 = a.sig2 * inv_r2;
    const float s6 = s2 * s2 * s2;
    // LJ: F_ij = g r_ij, g = 24 eps / r^2 (2 s^12 - s^6); 2 dg/d(r^2) below
    const float base = inv_r2 * s6;
    float g = a.eps24 * base * (2.0f * s6 - 1.0f);
    float gp = a.eps24 * base * inv_r2 * (8.0f - 28.0f * s6);
    const float gr = gi.x * dx + gi.y * dy + gi.z * dz;
    eacc += 24.0f * base * (2.0f * s6 - 1.0f) * gr;  // dF/deps (per unit eps)
    sacc += base * (24.0f * s6 - 6.0f) * gr;          // dF/dsigma / (24 eps / sigma)
    if (COUL) {
        float inv_r = rsqrtf(r2);
        inv_r = inv_r * (1.5f - 0.5f * r2 * inv_r * inv_r);
        const float gc = a.kc * __int_as_float(ri.w) * __int_as_float(rj.w) * inv_r * inv_r2;
        g += gc;
        gp -= 3.0f * gc * inv_r2;
    }
    const float ex = gi.x - gj.x, ey = gi.y - gj.y, ez = gi.z - gj.z;
    const float rd = gp * (dx * ex + dy * ey + dz * ez);
    hv.x += g * ex + rd * dx;
    hv.y += g * ey + rd * dy;
    hv.z += g * ez + rd * dz;
}

// Fixed-order block sum of two values over NT threads; thread 0 adds them to
// this block's partials (one writer per block and launches in stream order:
// deterministic).
template <int NT>
__device__ __forceinline__ void block_add2(double v0, double v1, double* part) {
    __shared__ double s[2][NT / 32];
    for (int sh = 16; sh > 0; sh >>= 1) {
        v0 += __shfl_xor_sync(0xffffffffu, v0, sh);
        v1 += __shfl_xor_sync(0xffffffffu, v1, sh);
    }
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { s[0][warp] = v0; s[1][warp] = v1; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0;
        for (int w = 0; w < NT / 32; ++w) { t0 += s[0][w]; t1 += s[1][w]; }
        part[2 * blockIdx.x] += t0;
        part[2 * blockIdx.x + 1] += t1;
    }
}

// Prepare the adjoints of the previous step from the adjoints (lx, lu) of this
// step's positions and velocities: a = (1 - M) lx, g = (1 - 2M) lu + dt a,
// M from x_t at the walls.
__device__ __forceinline__ void adj_prepare(const AdjArgs& a, int64_t i, const double lx[3],
                                            const double lu[3]) {
    float4 g4;
    float* gf = &g4.x;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double xv = a.xt[d][i];
        const bool M = (xv == a.lo[d]) || (xv == a.hi[d]);
        const double ab = M ? 0.0 : lx[d];
        const double g = (M ? -lu[d] : lu[d]) + a.dt * ab;
        a.abar[d][i] = ab;
        a.gd[d][i] = g;
        gf[d] = (float)g;
    }
    g4.w = 0.0f;
    a.g4_out[i] = g4;
}

// One reverse step.  One block per 256 atoms and kAdjTPA threads per atom:
// the forward step's union is staged (the step's fixed-point position records
// and the Float32 velocity adjoints), thread p of an atom gathers over list
// slots p, p + kAdjTPA, ..., and the slices are added in a fixed order.
template <bool COUL>
__global__ void __launch_bounds__(kBlock * kAdjTPA) k_adj_reverse(AdjArgs a) {
    extern __shared__ int4 adj_smem[];
    int4* srec = adj_smem;
    float4* sg = reinterpret_cast<float4*>(adj_smem + a.smrec);
    __shared__ float spart[kAdjTPA - 1][5][kBlock];
    const int tid = threadIdx.x;
    const int al = tid & (kBlock - 1);  // atom within the block
    const int part = tid / kBlock;      // list slice
    int64_t i = (int64_t)blockIdx.x * kBlock + al;
    const bool valid = i < a.n;
    const int32_t* __restrict__ U = a.ulist + (int64_t)blockIdx.x * a.ucap;
    {
        const int32_t nu = min(__ldg(&a.ucount[blockIdx.x]), a.ucap);
        const int32_t m = min(nu * a.apl, a.smrec);
        for (int32_t k = tid; k < m; k += kBlock * kAdjTPA) {
            const int64_t at = adj_atom(U, k, a.apl);
            srec[k] = __ldg(&a.recs[at]);
            sg[k] = a.g4_in[at];
        }
    }
    __syncthreads();
    if (!valid) i = a.n - 1;
    const int4 ri = __ldg(&a.recs[i]);
    const float4 gi = a.g4_in[i];
    const int32_t cpk = valid ? __ldg(&a.ncount[i]) : 0;
    const int32_t cnt = list_total(cpk);
    const uint16_t* __restrict__ L = a.llist + (int64_t)blockIdx.x * a.lcap * kBlock;
    float3 hv = make_float3(0.f, 0.f, 0.f);
    float eacc = 0.f, sacc = 0.f;
    int32_t li = part < cnt ? L[llist_at(list_slot(part, cpk, a.lcap), al)] : 0;
    for (int32_t s = part; s < cnt; s += kAdjTPA) {
        const int32_t sn = s + kAdjTPA;
        const int32_t next = sn < cnt ? L[llist_at(list_slot(sn, cpk, a.lcap), al)] : 0;
        int4 rj;
        float4 gj;
        if (li < a.smrec) {
            rj = srec[li];
            gj = sg[li];
        } else {
            const int64_t at = adj_atom(U, li, a.apl);
            rj = __ldg(&a.recs[at]);
            gj = a.g4_in[at];
        }
        hvp_pair<COUL>(a, ri, gi, rj, gj, hv, eacc, sacc);
        li = next;
    }
    if (part > 0) {
        spart[part - 1][0][al] = hv.x;
        spart[part - 1][1][al] = hv.y;
        spart[part - 1][2][al] = hv.z;
        spart[part - 1][3][al] = eacc;
        spart[part - 1][4][al] = sacc;
    }
    __syncthreads();
    double te = 0.0, ts = 0.0;
    if (part == 0 && valid) {
#pragma unroll
        for (int p = 0; p < kAdjTPA - 1; ++p) {
            hv.x += spart[p][0][al];
            hv.y += spart[p][1][al];
            hv.z += spart[p][2][al];
            eacc += spart[p][3][al];
            sacc += spart[p][4][al];
        }
        const double k = a.ckdt * a.im[i];
        const double lx[3] = {a.abar[0][i] + k * (double)hv.x, a.abar[1][i] + k * (double)hv.y,
                              a.abar[2][i] + k * (double)hv.z};
        const double lu[3] = {a.gd[0][i], a.gd[1][i], a.gd[2][i]};
        te = k * (double)eacc;
        ts = k * a.sfac * (double)sacc;
        if (a.last) {
#pragma unroll
            for (int d = 0; d < 3; ++d) { a.lx0[d][i] = lx[d]; a.lv0[d][i] = lu[d]; }
        } else {
            adj_prepare(a, i, lx, lu);
        }
    }
    block_add2<kBlock * kAdjTPA>(ts, te, a.gpart);
}

// Smooth pair weight of the histogram: 1 below r_switch, C2 switch to 0 at r_max.
__device__ __forceinline__ void hist_switch(const AdjArgs& a, float r, float& sw, float& dsw) {
    sw = 1.0f;
    dsw = 0.0f;
    if (r > a.rsw) {
        const float t = (r - a.rsw) * a.inv_span;
        const float t2 = t * t;
        sw = 1.0f - t2 * t * (10.0f - 15.0f * t + 6.0f * t2);
        dsw = -30.0f * t2 * (1.0f - t) * (1.0f - t) * a.inv_span;
    }
}

// Per-atom histogram rows of x_t (each unordered pair once: partners later in
// sorted order), kHistChunk bins per pass over the list.
__global__ void __launch_bounds__(kBlock) k_adj_hist(AdjArgs a) {
    const int tid = threadIdx.x;
    const int64_t i = (int64_t)blockIdx.x * kBlock + tid;
    if (i >= a.n) return;
    const int32_t* __restrict__ U = a.ulist + (int64_t)blockIdx.x * a.ucap;
    const int4 ri = __ldg(&a.recs[i]);
    const int32_t cpk = __ldg(&a.ncount[i]);
    const int32_t cnt = list_total(cpk);
    const uint16_t* __restrict__ L = a.llist + (int64_t)blockIdx.x * a.lcap * kBlock;
    for (int32_t b0 = 0; b0 < a.bins; b0 += kHistChunk) {
        float acc[kHistChunk];
#pragma unroll
        for (int k = 0; k < kHistChunk; ++k) acc[k] = 0.0f;
        for (int32_t s = 0; s < cnt; ++s) {
            const int64_t j = adj_atom(U, L[llist_at(list_slot(s, cpk, a.lcap), tid)], a.apl);
            if (j <= i) continue;
            const int4 rj = __ldg(&a.recs[j]);
            const float dx = (float)idiff(ri.x, rj.x) * a.invS;
            const float dy = (float)idiff(ri.y, rj.y) * a.invS;
            const float dz = (float)idiff(ri.z, rj.z) * a.invS;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 < a.rmax2)) continue;
            const float r = sqrtf(r2);
            float sw, dsw;
            hist_switch(a, r, sw, dsw);
#pragma unroll
            for (int k = 0; k < kHistChunk; ++k) {
                const float u = r - ((float)(b0 + k) + 0.5f) * a.bw;
                acc[k] += sw * expf(-u * u * a.inv2w2);
            }
        }
#pragma unroll
        for (int k = 0; k < kHistChunk; ++k)
            if (b0 + k < a.bins) a.hatom[(int64_t)(b0 + k) * a.n + i] = acc[k];
    }
}

// h_b = (1/N) sum over atoms of row b, fixed-order reduction (one block per bin).
__global__ void __launch_bounds__(256) k_adj_hist_reduce(const float* __restrict__ hatom,
                                                         int32_t n, double* __restrict__ h) {
    __shared__ double s[256];
    const float* row = hatom + (int64_t)blockIdx.x * n;
    double t = 0.0;
    for (int32_t k = threadIdx.x; k < n; k += 256) t += (double)row[k];
    s[threadIdx.x] = t;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) h[blockIdx.x] = s[0] / (double)n;
}

// Loss L = sum_b (h_b - target_b)^2 and the terminal coefficients 2 (h_b - t_b) / N.
__global__ void k_adj_loss(const double* __restrict__ h, const double* __restrict__ target,
                           int32_t bins, int32_t n, double* __restrict__ loss,
                           float* __restrict__ cb) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double L = 0.0;
    for (int32_t b = 0; b < bins; ++b) {
        const double e = h[b] - target[b];
        L += e * e;
        cb[b] = (float)(2.0 * e / (double)n);
    }
    *loss = L;
}

// dL/dx_K from the histogram (per atom over its whole list) and the adjoints
// of the last step.
__global__ void __launch_bounds__(kBlock) k_adj_terminal(AdjArgs a) {
    extern __shared__ float scb[];
    const int tid = threadIdx.x;
    for (int32_t b = tid; b < a.bins; b += kBlock) scb[b] = a.cb[b];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * kBlock + tid;
    if (i >= a.n) return;
    const int32_t* __restrict__ U = a.ulist + (int64_t)blockIdx.x * a.ucap;
    const int4 ri = __ldg(&a.recs[i]);
    const int32_t cpk = __ldg(&a.ncount[i]);
    const int32_t cnt = list_total(cpk);
    const uint16_t* __restrict__ L = a.llist + (int64_t)blockIdx.x * a.lcap * kBlock;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for (int32_t s = 0; s < cnt; ++s) {
        const int64_t j = adj_atom(U, L[llist_at(list_slot(s, cpk, a.lcap), tid)], a.apl);
        const int4 rj = __ldg(&a.recs[j]);
        const float dx = (float)idiff(ri.x, rj.x) * a.invS;
        const float dy = (float)idiff(ri.y, rj.y) * a.invS;
        const float dz = (float)idiff(ri.z, rj.z) * a.invS;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (!(r2 < a.rmax2)) continue;
        const float r = sqrtf(r2);
        float sw, dsw;
        hist_switch(a, r, sw, dsw);
        float c = 0.0f;
        for (int32_t b = 0; b < a.bins; ++b) {
            const float u = r - ((float)b + 0.5f) * a.bw;
            const float e = expf(-u * u * a.inv2w2);
            c += scb[b] * e * (dsw - sw * u * a.invw2);
        }
        c /= r;
        gx += c * dx;
        gy += c * dy;
        gz += c * dz;
    }
    const double lx[3] = {(double)gx, (double)gy, (double)gz};
    const double lu[3] = {0.0, 0.0, 0.0};
    adj_prepare(a, i, lx, lu);
}

// Undo a re-sort on the adjoints: old[perm[k]] = new[k].
__global__ void k_adj_unpermute(const int32_t* __restrict__ perm, int32_t n,
                                const double* __restrict__ src, double* __restrict__ dst,
                                const float4* __restrict__ g4src, float4* __restrict__ g4dst) {
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int32_t o = perm[k];
#pragma unroll
    for (int c = 0; c < 6; ++c) dst[(int64_t)c * n + o] = src[(int64_t)c * n + k];
    g4dst[o] = g4src[k];
}

// Sorted -> caller order for the gradients (N x 3 interleaved each).
__global__ void k_adj_unsort(const int32_t* __restrict__ orig, int32_t n,
                             const double* __restrict__ lx, const double* __restrict__ lv,
                             double* __restrict__ dx, double* __restrict__ dv) {
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t o = orig[k];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dx[3 * o + d] = lx[(int64_t)d * n + k];
        dv[3 * o + d] = lv[(int64_t)d * n + k];
    }
}

__global__ void k_adj_gpar(const double* __restrict__ part, int32_t nb, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0, e = 0.0;
    for (int32_t b = 0; b < nb; ++b) { s += part[2 * b]; e += part[2 * b + 1]; }
    out[0] = s;
    out[1] = e;
}


// Marks an early refit taken after step t (runs inside the refit's conditional body).
__global__ void k_adj_flag(uint8_t* flags, int32_t t) {
    if (threadIdx.x == 0 && blockIdx.x == 0) flags[t] = 1;
}

// ------------------------------------------------------------------ driver
//
// Schedule of one trajectory (t = 0 .. K-1, step t moves x_t to x_{t+1}):
//   t % C == 0   checkpoint (the state before anything else at t)
//   t % Q == 0   re-sort (Q = resort_every * R; C is a multiple of Q), the
//                permutation and the sorted codes kept for the reverse pass
//   t % R == 0   otherwise: refit
//   after step t, inside a window: an early refit when the step kernel finds
//   an atom that could pass skin/2 in the next step -- decided on the device
//   in the forward pass (a conditional graph node that also records the
//   decision), replayed from the record in the backward pass.

struct AdjEngine {
    Ctx* parent = nullptr;
    MDEngine* m = nullptr;
    nd_adj_spec s{};
    int32_t n = 0, K = 0, C = 0, R = 0, Q = 0, nseg = 0, nsort = 0;
    int32_t smrec = 0;
    size_t rev_smem = 0, ckpt_bytes = 0;
    DevBuf ckpt, perms, codes, statics, traj, trajrec, recK, lam, lam_tmp, g4[2], gpart, xK, hatom, hist, target,
        cb, scal, outs, flags;
    bool timed[2] = {false, false};  // forward / backward events recorded
    bool have_forward = false;
    std::vector<uint8_t> sched;      // early refits after step t (last forward pass)
    std::vector<uint8_t> sched_bwd;  // the schedule the backward graph was captured with
    cudaGraphExec_t g_fwd = nullptr, g_bwd = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
};

static double* lam_p(AdjEngine* A) { return (double*)A->lam.p; }

static bool adj_coulomb(const AdjEngine* A) {
    return A->m->has_q && A->m->p.coulomb_k != 0.0;
}

static AdjArgs adj_args(AdjEngine* A, const double* xt, const int4* recs) {
    MDEngine* m = A->m;
    AdjArgs a{};
    a.n = m->n;
    a.apl = m->apl;
    a.ucap = m->ucap;
    a.smrec = A->smrec;
    a.ulist = (const int32_t*)m->ulist.p;
    a.ucount = (const int32_t*)m->ucount.p;
    a.llist = (const uint16_t*)m->llist.p;
    a.ncount = (const int32_t*)m->ncount.p;
    a.lcap = m->lcap;
    const size_t n = (size_t)m->n;
    for (int d = 0; d < 3; ++d) a.xt[d] = xt + d * n;
    a.recs = recs;
    a.im = m->set[0].im;
    double* L = lam_p(A);
    for (int d = 0; d < 3; ++d) {
        a.abar[d] = L + d * n;
        a.gd[d] = L + (3 + d) * n;
        a.lx0[d] = (double*)A->outs.p + d * n;
        a.lv0[d] = (double*)A->outs.p + (3 + d) * n;
    }
    a.gpart = (double*)A->gpart.p;
    for (int d = 0; d < 3; ++d) {
        a.lo[d] = m->p.box_lo[d];
        a.hi[d] = m->p.box_hi[d];
    }
    a.invS = (float)(1.0 / m->fr.s);
    const nd_md_params& p = m->p;
    a.rc2 = (float)(p.cutoff * p.cutoff);
    a.sig2 = (float)(p.sigma * p.sigma);
    a.eps24 = (float)(24.0 * p.epsilon);
    a.kc = (float)p.coulomb_k;
    a.sfac = 24.0 * p.epsilon / p.sigma;
    a.dt = p.dt;
    a.bins = A->s.bins;
    a.rmax2 = (float)(A->s.r_max * A->s.r_max);
    a.bw = (float)(A->s.r_max / A->s.bins);
    a.inv2w2 = (float)(1.0 / (2.0 * A->s.width * A->s.width));
    a.invw2 = (float)(1.0 / (A->s.width * A->s.width));
    a.rsw = (float)A->s.r_switch;
    a.inv_span = (float)(1.0 / (A->s.r_max - A->s.r_switch));
    a.hatom = (float*)A->hatom.p;
    a.cb = (const float*)A->cb.p;
    a.err = m->sub.d_err;
    return a;
}

static double* live_set(AdjEngine* A) { return (double*)A->m->set_buf[0].p; }

// The per-atom fields a re-sort permutes besides x and u: q and 1/m (FP64)
// and the original index (int32), contiguous in the state set.
static void* adj_statics(AdjEngine* A) { return live_set(A) + 6 * (size_t)A->n; }
static size_t adj_statics_bytes(const AdjEngine* A) {
    return (size_t)A->n * (2 * sizeof(double) + sizeof(int32_t));
}

static nd_status adj_copy(AdjEngine* A, void* dst, const void* src, size_t bytes, const char* what) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, A->m->sub.stream);
    if (e != cudaSuccess) return cuda_fail(&A->m->sub, e, what);
    return ND_OK;
}

// One forward step of the engine (records ping-pong as in the plain engine).
static void adj_step(AdjEngine* A, bool first, int use_cond = 0,
                     cudaGraphConditionalHandle h = 0, int unchecked = 0) {
    MDEngine* m = A->m;
    StepArgs a = md_step_args(m, m->rc);
    a.use_cond = use_cond;
    a.vote = use_cond;
    a.unchecked = unchecked;
    a.cond = h;
    md_launch_step(m, a, first);
    m->rc ^= 1;
}

// Whether an early refit may follow step t: after the window's steps 0, M,
// 2M, ... (M = the engine's check interval), not before a scheduled rebuild.
static bool adj_cond_after(const AdjEngine* A, int32_t t) {
    return (t + 1) % A->R != 0 && t + 1 < A->K && (t % A->R) % A->m->check_every == 0;
}

// Rebuild before step t of the static schedule (re-sort, refit, or the early
// refit recorded after step t-1).  keep: save the re-sort's permutation and
// codes (forward pass).
static nd_status adj_rebuild_before(AdjEngine* A, int32_t t, bool keep) {
    MDEngine* m = A->m;
    nd_status st;
    const size_t n = (size_t)A->n;
    if (t % A->Q == 0) {
        if ((st = md_rebuild(m, RB_RESORT))) return st;
        if (!keep) return ND_OK;
        const int32_t k = t / A->Q;
        if ((st = adj_copy(A, (int32_t*)A->perms.p + k * n, m->sub.perm.p, sizeof(int32_t) * n, "perm")))
            return st;
        if ((st = adj_copy(A, (int32_t*)A->codes.p + k * n, m->sub.codes.p, sizeof(int32_t) * n, "codes")))
            return st;
        return adj_copy(A, (char*)A->statics.p + k * adj_statics_bytes(A), adj_statics(A),
                        adj_statics_bytes(A), "charges, masses, indices");
    }
    if (t % A->R == 0) return md_rebuild(m, RB_REFIT);
    return ND_OK;
}

// Forward pass: K steps from checkpoint 0 with device-decided early refits,
// checkpoints, permutations and codes saved, then the histogram of x_K and
// the loss.
static nd_status adj_enqueue_forward(AdjEngine* A) {
    MDEngine* m = A->m;
    Ctx* c = &m->sub;
    nd_status st;
    const size_t n = (size_t)A->n;
    char* ck = (char*)A->ckpt.p;
    cudaMemsetAsync(m->diag.p, 0, sizeof(unsigned long long), c->stream);
    cudaMemsetAsync(A->flags.p, 0, (size_t)A->K, c->stream);
    for (int32_t t = 0; t < A->K; ++t) {
        if (t % A->C == 0) {
            const int32_t sg = t / A->C;
            st = t == 0 ? adj_copy(A, live_set(A), ck, A->ckpt_bytes, "restore")
                        : adj_copy(A, ck + sg * A->ckpt_bytes, live_set(A), A->ckpt_bytes, "checkpoint");
            if (st) return st;
        }
        if ((st = adj_rebuild_before(A, t, true))) return st;
        const bool cond = adj_cond_after(A, t);
        cudaGraphConditionalHandle h = 0;
        if (cond && (st = md_cond_handle(m, &h))) return st;
        // the list is used unchecked after this step when no check follows
        // and no scheduled rebuild comes first (the loss at x_K included)
        const bool unchecked = !cond && ((t + 1) % A->R != 0 || t + 1 == A->K);
        adj_step(A, t == 0, cond ? 1 : 0, h, unchecked ? 1 : 0);
        if (cond &&
            (st = md_add_cond_node(m, h, 1, [&](int) {
                 nd_status s2 = md_rebuild(m, RB_REFIT, m->rc);
                 if (s2 == ND_OK) {
                     k_adj_flag<<<1, 32, 0, m->sub.stream>>>((uint8_t*)A->flags.p, t);
                     m->sub.launches++;
                 }
                 return s2;
             })))
            return st;
    }
    if ((st = adj_copy(A, A->xK.p, live_set(A), 3 * sizeof(double) * n, "x_K")) ||
        (st = adj_copy(A, A->recK.p, m->rec_buf[m->rc].p, sizeof(int4) * n, "x_K records")))
        return st;
    AdjArgs a = adj_args(A, (const double*)A->xK.p, (const int4*)A->recK.p);
    const unsigned nb = (unsigned)m->nblocks;
    k_adj_hist<<<nb, kBlock, 0, c->stream>>>(a);
    k_adj_hist_reduce<<<(unsigned)A->s.bins, 256, 0, c->stream>>>((const float*)A->hatom.p, A->n,
                                                                   (double*)A->hist.p);
    k_adj_loss<<<1, 32, 0, c->stream>>>((const double*)A->hist.p, (const double*)A->target.p,
                                        A->s.bins, A->n, (double*)A->scal.p, (float*)A->cb.p);
    c->launches += 3;
    return check_launch(c, "adjoint forward");
}

// Backward pass: the terminal adjoint at x_K, then every segment (last first)
// is recomputed from its checkpoint on the recorded schedule and reversed
// list epoch by list epoch (an epoch runs from one rebuild to the next).
static nd_status adj_enqueue_backward(AdjEngine* A) {
    MDEngine* m = A->m;
    Ctx* c = &m->sub;
    nd_status st;
    const size_t n = (size_t)A->n;
    const unsigned nb = (unsigned)m->nblocks;
    const unsigned g256 = (unsigned)cdiv(A->n, 256);
    char* ck = (char*)A->ckpt.p;
    double* traj = (double*)A->traj.p;
    int4* trec = (int4*)A->trajrec.p;
    const std::vector<uint8_t>& sched = A->sched;
    cudaMemsetAsync(A->gpart.p, 0, 2 * sizeof(double) * nb, c->stream);
    int gc = 0;  // g4 buffer holding g of the next reverse step
    {
        AdjArgs a = adj_args(A, (const double*)A->xK.p, (const int4*)A->recK.p);
        a.g4_out = (float4*)A->g4[gc].p;
        k_adj_terminal<<<nb, kBlock, sizeof(float) * (size_t)A->s.bins, c->stream>>>(a);
        c->launches++;
    }
    for (int32_t sg = A->nseg - 1; sg >= 0; --sg) {
        const int32_t t0 = sg * A->C;
        if ((st = adj_copy(A, live_set(A), ck + sg * A->ckpt_bytes, A->ckpt_bytes, "restore"))) return st;
        for (int32_t k = 0; k < A->C; ++k) {
            const int32_t t = t0 + k;
            if ((st = adj_rebuild_before(A, t, false))) return st;
            if (t % A->R != 0 && sched[t - 1] && (st = md_rebuild(m, RB_REFIT, m->rc))) return st;
            if ((st = adj_copy(A, traj + k * 3 * n, live_set(A), 3 * sizeof(double) * n, "trajectory")) ||
                (st = adj_copy(A, trec + k * n, m->rec_buf[m->rc].p, sizeof(int4) * n, "records")))
                return st;
            if (k < A->C - 1) adj_step(A, t == 0);
        }
        for (int32_t a0 = t0 + A->C - A->Q; a0 >= t0; a0 -= A->Q) {
            // this stretch's order: its sorted codes (the tree of its refits)
            // and its charges, inverse masses and original indices
            if (a0 != t0 + A->C - A->Q &&
                ((st = adj_copy(A, c->codes.p, (int32_t*)A->codes.p + (a0 / A->Q) * n,
                                sizeof(int32_t) * n, "codes")) ||
                 (st = adj_copy(A, adj_statics(A),
                                (char*)A->statics.p + (a0 / A->Q) * adj_statics_bytes(A),
                                adj_statics_bytes(A), "charges, masses, indices"))))
                return st;
            int32_t e = a0 + A->Q;
            for (int32_t s = e - 1; s >= a0; --s) {
                const bool start = s == a0 || s % A->R == 0 || sched[s - 1];
                if (!start) continue;
                if ((st = adj_copy(A, live_set(A), traj + (s - t0) * 3 * n, 3 * sizeof(double) * n,
                                   "epoch")))
                    return st;
                if ((st = md_rebuild(m, RB_REFIT))) return st;
                for (int32_t t = e - 1; t >= s; --t) {
                    AdjArgs a = adj_args(A, traj + (t - t0) * 3 * n, trec + (t - t0) * n);
                    a.g4_in = (const float4*)A->g4[gc].p;
                    a.g4_out = (float4*)A->g4[gc ^ 1].p;
                    a.ckdt = (t == 0 ? 0.5 : 1.0) * m->p.dt;
                    a.last = t == 0 ? 1 : 0;
                    const unsigned nt = kBlock * kAdjTPA;
                    if (adj_coulomb(A)) k_adj_reverse<true><<<nb, nt, A->rev_smem, c->stream>>>(a);
                    else k_adj_reverse<false><<<nb, nt, A->rev_smem, c->stream>>>(a);
                    c->launches++;
                    gc ^= 1;
                }
                e = s;
            }
            if (a0 > 0) {
                k_adj_unpermute<<<g256, 256, 0, c->stream>>>(
                    (const int32_t*)A->perms.p + (a0 / A->Q) * n, A->n, lam_p(A),
                    (double*)A->lam_tmp.p, (const float4*)A->g4[gc].p, (float4*)A->g4[gc ^ 1].p);
                c->launches++;
                gc ^= 1;
                if ((st = adj_copy(A, lam_p(A), A->lam_tmp.p, 6 * sizeof(double) * n, "unpermute")))
                    return st;
            }
        }
    }
    // segment 0 after its opening re-sort is in creation order: its original
    // indices unsort the gradients
    const double* outs = (const double*)A->outs.p;
    k_adj_unsort<<<g256, 256, 0, c->stream>>>(m->set[0].orig, A->n, outs, outs + 3 * n,
                                              (double*)A->outs.p + 6 * n,
                                              (double*)A->outs.p + 9 * n);
    k_adj_gpar<<<1, 32, 0, c->stream>>>((const double*)A->gpart.p, (int32_t)nb,
                                        (double*)A->scal.p + 1);
    c->launches += 2;
    return check_launch(c, "adjoint backward");
}

// Capture one pass into a graph (instantiated once per setting).
template <class F>
static nd_status adj_capture(AdjEngine* A, cudaGraphExec_t* out, F&& body) {
    Ctx* c = &A->m->sub;
    cudaGraph_t g = nullptr;
    const int64_t l0 = c->launches;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(c, e, "begin capture");
    nd_status st = body();
    e = cudaStreamEndCapture(c->stream, &g);
    c->launches = l0;
    if (st) { if (g) cudaGraphDestroy(g); return st; }
    if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "graph instantiate");
    return ND_OK;
}

static void adj_drop_graphs(AdjEngine* A) {
    if (A->g_fwd) cudaGraphExecDestroy(A->g_fwd);
    if (A->g_bwd) cudaGraphExecDestroy(A->g_bwd);
    A->g_fwd = A->g_bwd = nullptr;
}

nd_status adj_destroy(AdjEngine* A) {
    if (!A) return ND_OK;
    if (A->m) cudaStreamSynchronize(A->m->sub.stream);
    adj_drop_graphs(A);
    for (cudaEvent_t e : A->ev)
        if (e) cudaEventDestroy(e);
    DevBuf* bufs[] = {&A->ckpt, &A->perms, &A->codes, &A->statics, &A->traj, &A->trajrec, &A->recK, &A->lam, &A->lam_tmp, &A->g4[0],
                      &A->g4[1], &A->gpart, &A->xK, &A->hatom, &A->hist, &A->target, &A->cb,
                      &A->scal, &A->outs, &A->flags};
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    if (A->m) md_destroy(A->m);
    delete A;
    return ND_OK;
}

nd_status adj_create(Ctx* parent, const nd_md_params* p, int32_t n, const double* x0,
                     const double* v0, const double* q, const double* mass, const nd_adj_spec* s,
                     AdjEngine** out) {
    if (!parent || !p || !s || !out || !x0 || !v0 || n <= 1) return ND_ERR_ARG;
    nd_adj_spec sp = *s;
    if (sp.checkpoint_every <= 0) sp.checkpoint_every = 50;
    if (sp.bins <= 0 || sp.bins > 1024 || !(sp.r_max > 0) || sp.r_max > p->cutoff) return ND_ERR_ARG;
    if (!(sp.width > 0)) sp.width = sp.r_max / sp.bins;
    if (sp.r_switch < 0) sp.r_switch = sp.r_max - std::min(0.25, 0.5 * sp.r_max);
    if (!(sp.r_switch < sp.r_max)) return ND_ERR_ARG;
    const int32_t R = p->rebuild_every;
    const int32_t Q = (p->resort_every > 0 ? p->resort_every : 5) * std::max(R, 1);
    if (R <= 0 || sp.steps <= 0 || sp.checkpoint_every % Q || sp.steps % sp.checkpoint_every)
        return ND_ERR_ARG;
    if (!(p->sigma > 0)) return ND_ERR_ARG;
    AdjEngine* A = new AdjEngine();
    A->parent = parent;
    A->s = sp;
    A->n = n;
    A->K = sp.steps;
    A->C = sp.checkpoint_every;
    A->R = R;
    A->Q = Q;
    A->nseg = A->K / A->C;
    A->nsort = A->K / A->Q;
    nd_status st = md_create(parent, p, n, x0, v0, q, mass, true, false, &A->m);
    if (st) { delete A; return st; }
    MDEngine* m = A->m;
    Ctx* c = &m->sub;
    const size_t nn = (size_t)n;
    A->ckpt_bytes = nn * (8 * sizeof(double) + sizeof(int32_t));
    A->ckpt_bytes = (A->ckpt_bytes + 255) / 256 * 256;
    int maxsm = 0;
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
    // dynamic: 32 B per staged union atom; static: the slice partials and the
    // block reduction
    const int static_sm = (int)(sizeof(float) * 5 * kBlock * (kAdjTPA - 1)) + 2048;
    A->smrec = std::max(0, std::min(m->ucap_sm * m->apl, (maxsm - static_sm) / 32));
    A->rev_smem = 32 * (size_t)A->smrec;
    cudaError_t e = cudaFuncSetAttribute((const void*)k_adj_reverse<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)A->rev_smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute((const void*)k_adj_reverse<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)A->rev_smem);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { st = cuda_fail(parent, e, "adjoint setup"); adj_destroy(A); return st; }
    if ((st = ensure(c, A->ckpt, A->ckpt_bytes * A->nseg)) ||
        (st = ensure(c, A->perms, sizeof(int32_t) * nn * A->nsort)) ||
        (st = ensure(c, A->codes, sizeof(int32_t) * nn * A->nsort)) ||
        (st = ensure(c, A->statics, adj_statics_bytes(A) * A->nsort)) ||
        (st = ensure(c, A->traj, 3 * sizeof(double) * nn * A->C)) ||
        (st = ensure(c, A->trajrec, sizeof(int4) * nn * A->C)) ||
        (st = ensure(c, A->recK, sizeof(int4) * nn)) ||
        (st = ensure(c, A->lam, 6 * sizeof(double) * nn)) ||
        (st = ensure(c, A->lam_tmp, 6 * sizeof(double) * nn)) ||
        (st = ensure(c, A->g4[0], sizeof(float4) * nn)) ||
        (st = ensure(c, A->g4[1], sizeof(float4) * nn)) ||
        (st = ensure(c, A->gpart, 2 * sizeof(double) * (size_t)m->nblocks)) ||
        (st = ensure(c, A->xK, 3 * sizeof(double) * nn)) ||
        (st = ensure(c, A->hatom, sizeof(float) * nn * (size_t)sp.bins)) ||
        (st = ensure(c, A->hist, sizeof(double) * (size_t)sp.bins)) ||
        (st = ensure(c, A->target, sizeof(double) * (size_t)sp.bins)) ||
        (st = ensure(c, A->cb, sizeof(float) * (size_t)sp.bins)) ||
        (st = ensure(c, A->scal, 4 * sizeof(double))) ||
        (st = ensure(c, A->outs, 12 * sizeof(double) * nn)) ||
        (st = ensure(c, A->flags, (size_t)A->K))) {
        parent->last_error = c->last_error;
        adj_destroy(A);
        return st;
    }
    cudaMemsetAsync(A->target.p, 0, sizeof(double) * (size_t)sp.bins, c->stream);
    for (cudaEvent_t& ev : A->ev)
        if (cudaEventCreate(&ev) != cudaSuccess) {
            st = cuda_fail(parent, cudaGetLastError(), "adjoint events");
            adj_destroy(A);
            return st;
        }
    // checkpoint 0 := the engine's state after its opening sort
    if ((st = adj_copy(A, A->ckpt.p, live_set(A), A->ckpt_bytes, "initial checkpoint")) ||
        (st = sync_and_check(c, "adjoint setup"))) {
        parent->last_error = c->last_error;
        adj_destroy(A);
        return st;
    }
    *out = A;
    return ND_OK;
}

nd_status adj_set_params(AdjEngine* A, double sigma, double epsilon) {
    if (!(sigma > 0) || !std::isfinite(epsilon)) return ND_ERR_ARG;
    A->m->p.sigma = sigma;
    A->m->p.epsilon = epsilon;
    adj_drop_graphs(A);
    A->have_forward = false;
    return ND_OK;
}

nd_status adj_set_target(AdjEngine* A, const double* target) {
    Ctx* c = &A->m->sub;
    cudaError_t e = target ? cudaMemcpyAsync(A->target.p, target, sizeof(double) * A->s.bins,
                                             cudaMemcpyHostToDevice, c->stream)
                           : cudaMemsetAsync(A->target.p, 0, sizeof(double) * A->s.bins, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint target");
    A->have_forward = false;
    return sync_and_check(c, "adjoint target");
}

nd_status adj_forward(AdjEngine* A, double* hist, double* loss) {
    NvtxRange nv("nd adjoint forward");
    MDEngine* m = A->m;
    Ctx* c = &m->sub;
    nd_status st;
    A->have_forward = false;
    if (!A->g_fwd && (st = adj_capture(A, &A->g_fwd, [&] { return adj_enqueue_forward(A); })))
        return st;
    cudaEventRecord(A->ev[0], c->stream);
    cudaError_t e = cudaGraphLaunch(A->g_fwd, c->stream);
    cudaEventRecord(A->ev[1], c->stream);
    A->timed[0] = true;
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint forward");
    double sc[4];
    std::vector<double> h((size_t)A->s.bins);
    std::vector<uint8_t> sched((size_t)A->K);
    unsigned long long viol = 0;
    e = cudaMemcpyAsync(sc, A->scal.p, sizeof(sc), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), A->hist.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sched.data(), A->flags.p, sched.size(), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&viol, m->diag.p, sizeof(viol), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint forward");
    if ((st = sync_and_check(c, "adjoint forward"))) return st;
    if (viol) {
        c->last_error = "an atom moved more than skin/2 from its list-build position within "
                        "one step: raise skin or lower rebuild_every";
        return ND_ERR_OVERFLOW;
    }
    A->sched = std::move(sched);
    if (hist) std::copy(h.begin(), h.end(), hist);
    if (loss) *loss = sc[0];
    A->have_forward = true;
    return ND_OK;
}

nd_status adj_backward(AdjEngine* A, double* dx0, double* dv0, double* dsigma, double* deps) {
    NvtxRange nv("nd adjoint backward");
    MDEngine* m = A->m;
    Ctx* c = &m->sub;
    nd_status st;
    if (!A->have_forward) {
        c->last_error = "backward needs the forward pass of the current settings first";
        return ND_ERR_ARG;
    }
    // the backward graph replays the forward pass's early refits
    if (A->g_bwd && A->sched_bwd != A->sched) {
        cudaGraphExecDestroy(A->g_bwd);
        A->g_bwd = nullptr;
    }
    if (!A->g_bwd) {
        if ((st = adj_capture(A, &A->g_bwd, [&] { return adj_enqueue_backward(A); }))) return st;
        A->sched_bwd = A->sched;
    }
    cudaEventRecord(A->ev[2], c->stream);
    cudaError_t e = cudaGraphLaunch(A->g_bwd, c->stream);
    cudaEventRecord(A->ev[3], c->stream);
    A->timed[1] = true;
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint backward");
    const size_t n = (size_t)A->n;
    double sc[4];
    e = cudaMemcpyAsync(sc, A->scal.p, sizeof(sc), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && dx0)
        e = cudaMemcpyAsync(dx0, (double*)A->outs.p + 6 * n, 3 * sizeof(double) * n,
                            cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && dv0)
        e = cudaMemcpyAsync(dv0, (double*)A->outs.p + 9 * n, 3 * sizeof(double) * n,
                            cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint backward");
    // the pass moved the live state and lists: a new backward needs a new forward
    A->have_forward = false;
    if ((st = sync_and_check(c, "adjoint backward"))) return st;
    if (dsigma) *dsigma = sc[1];
    if (deps) *deps = sc[2];
    return ND_OK;
}

nd_status adj_times(AdjEngine* A, float* fwd_ms, float* bwd_ms) {
    Ctx* c = &A->m->sub;
    cudaError_t e = cudaSuccess;
    if (fwd_ms) *fwd_ms = -1.0f;
    if (bwd_ms) *bwd_ms = -1.0f;
    if (fwd_ms && A->timed[0]) e = cudaEventElapsedTime(fwd_ms, A->ev[0], A->ev[1]);
    if (e == cudaSuccess && bwd_ms && A->timed[1])
        e = cudaEventElapsedTime(bwd_ms, A->ev[2], A->ev[3]);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint times");
    return ND_OK;
}

nd_status adj_final(AdjEngine* A, double* x) {
    Ctx* c = &A->m->sub;
    if (!A->have_forward) {
        c->last_error = "no forward pass of the current settings";
        return ND_ERR_ARG;
    }
    // x_K in the live order -> caller order through the live set's indices
    const size_t n = (size_t)A->n;
    double* tmp = (double*)A->outs.p + 6 * n;
    const double* xk = (const double*)A->xK.p;
    k_adj_unsort<<<(unsigned)cdiv(A->n, 256), 256, 0, c->stream>>>(A->m->set[0].orig, A->n, xk,
                                                                   xk, tmp, tmp + 3 * n);
    cudaError_t e = cudaMemcpyAsync(x, tmp, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint final state");
    return sync_and_check(c, "adjoint final state");
}

const char* adj_last_error(AdjEngine* A) { return A->m->sub.last_error.c_str(); }

}  // namespace nd
