// nd_md.cu -- device-resident molecular dynamics for sm_103a: the GPU form of
// simulate! (src/Simulator.jl:154-256) with the intended physics of
// force_lennardjones! / force_coulomb! / sum_forces! (src/Forces.jl) and
// kick-drift-kick velocity Verlet with boundary_reflect! walls
// (src/Simulator.jl:81-111).
//
// Layout in HBM (atoms are kept in tree order and re-sorted at every rebuild):
//   x[3][N], w[3][N]   FP64 positions and velocities, one array per component
//                      (two sets, ping-ponged by the reorder at each rebuild)
//   q[N], im[N]        FP64 charge and inverse mass (optional)
//   sh[2N]             float4 shadow of x for the pair math, one 32-byte record
//                      per atom: sh[2k] = (hi, q) with hi = fl32(x), sh[2k+1] =
//                      (lo, 0) with lo = fl32(x - hi) (ping-ponged per step)
//   nbr[cap][N]        full neighbour list, slot-major (coalesced per slot)
//   f[N]               float4 forces of the last evaluation
// One MD step is ONE kernel: each thread owns an atom, sums its pair forces
// over its list (no atomics, deterministic), completes the pending half kick,
// kicks, drifts, reflects and writes the next shadow.  Velocities are stored
// at half steps between kernels (w = v_{n-1/2} after reflection).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "nd_internal.cuh"

namespace nd {

struct MDEngine;

// ------------------------------------------------------------- kernels

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

__device__ __forceinline__ void split_df(double x, float& hi, float& lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}

struct SetPtrs {
    double* x[3];
    double* w[3];
    double* q;
    double* im;
    int32_t* orig;
};

// Gather every per-atom array into the new (sorted) order and refresh the
// float shadows; pos32 keeps the Float32 positions used by the tree.
__global__ void k_md_reorder(SetPtrs src, SetPtrs dst, const int32_t* __restrict__ perm,
                             const float* __restrict__ xyz32, int32_t n, float4* __restrict__ pos32,
                             float4* __restrict__ sh) {
    int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int32_t o = perm[k];
    float h[3], l[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double xv = src.x[d][o];
        dst.x[d][k] = xv;
        dst.w[d][k] = src.w[d][o];
        split_df(xv, h[d], l[d]);
    }
    double qv = src.q[o];
    dst.q[k] = qv;
    dst.im[k] = src.im[o];
    dst.orig[k] = src.orig[o];
    pos32[k] = make_float4(xyz32[3 * (int64_t)o], xyz32[3 * (int64_t)o + 1],
                           xyz32[3 * (int64_t)o + 2], __int_as_float(k));
    sh[2 * (int64_t)k] = make_float4(h[0], h[1], h[2], (float)qv);
    sh[2 * (int64_t)k + 1] = make_float4(l[0], l[1], l[2], 0.0f);
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

// Full neighbour list: every atom walks the tree from the root with its own
// box (p -/+ h_q, h_q slightly above r_list/2 so the box test never drops a
// pair) and keeps the j != i with d^2 < r_list^2 (Float32, reference formula).
__global__ void __launch_bounds__(128)
    k_md_neighbors(const float4* __restrict__ keys, const float4* __restrict__ pos, int32_t n,
                   int32_t nL, int32_t apl, float hq, float rl2, int32_t cap,
                   int32_t* __restrict__ nbr, int32_t* __restrict__ ncount, int32_t* err) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = __ldg(&pos[i]);
    float qmnx = __fsub_rn(p.x, hq), qmny = __fsub_rn(p.y, hq), qmnz = __fsub_rn(p.z, hq);
    float qmxx = __fadd_rn(p.x, hq), qmxy = __fadd_rn(p.y, hq), qmxz = __fadd_rn(p.z, hq);
    int32_t cnt = 0;
    int32_t t = nL + 1;
    int64_t guard = 0;
    const int64_t max_visits = 4LL * nL + 8;
    while (t != 0) {
        if (++guard > max_visits || t < 1 || t > 2 * nL - 1) { set_error(err, ND_ERR_INTERNAL, i); break; }
        float4 a = __ldg(&keys[2 * (int64_t)(t - 1)]);
        float4 b = __ldg(&keys[2 * (int64_t)(t - 1) + 1]);
        int32_t left = __float_as_int(b.z), skip = __float_as_int(b.w);
        bool ov = (qmnx < a.w) & (qmxx > a.x) & (qmny < b.x) & (qmxy > a.y) & (qmnz < b.y) &
                  (qmxz > a.z);
        if (ov) {
            if (left == 0) {
                int64_t base = (int64_t)(t - 1) * apl;
                for (int32_t e = 0; e < apl; ++e) {
                    int32_t j = (int32_t)(base + e);
                    if (j == i) continue;
                    float4 q = __ldg(&pos[j]);
                    float d2 = dist2_ref(p.x, p.y, p.z, q.x, q.y, q.z);
                    if (d2 < rl2) {
                        if (cnt < cap) nbr[(int64_t)cnt * n + i] = j;
                        ++cnt;
                    }
                }
                t = skip;
            } else {
                t = left;
            }
        } else {
            t = skip;
        }
    }
    ncount[i] = min(cnt, cap);
    if (cnt > cap) set_error(err, ND_ERR_OVERFLOW, i);
    atomicMax(err + 2, cnt);
}

struct StepArgs {
    int32_t n;
    const int32_t* __restrict__ nbr;
    const int32_t* __restrict__ ncount;
    const float4* __restrict__ sh_in;  // interleaved (hi, lo) records
    float4* __restrict__ sh_out;
    double* x[3];
    double* w[3];
    const double* __restrict__ im;
    float4* __restrict__ f_out;
    double* __restrict__ v_out[3];  // measure kernel: integer-step velocity
    double* __restrict__ acc;       // measure kernel: [0] potential, [1] kinetic
    const float4* __restrict__ pos_build;  // Float32 positions at the last rebuild
    unsigned long long* __restrict__ diag; // [0] atom-steps that moved > skin/2 since the build
    float half_skin2;
    float rc2, sig2, eps24, eps4, kc;
    float hdt;                      // dt / 2
    double dt;
    double lo[3], hi[3];
};

// LJ + Coulomb pair force magnitude over r (F_ij = fmag * r_ij) and energy.
template <bool COUL, bool ENERGY>
__device__ __forceinline__ void pair_lj_coul(float r2, float qq, const StepArgs& a, float& fmag,
                                             float& u) {
    float inv_r2 = __frcp_rn(r2);
    float s2 = a.sig2 * inv_r2;
    float s6 = s2 * s2 * s2;
    fmag = a.eps24 * inv_r2 * s6 * (2.0f * s6 - 1.0f);
    if (ENERGY) u = a.eps4 * s6 * (s6 - 1.0f);
    if (COUL) {
        float inv_r = rsqrtf(r2);
        inv_r = inv_r * (1.5f - 0.5f * r2 * inv_r * inv_r);  // one Newton step
        float e = a.kc * qq * inv_r;
        fmag += e * inv_r2;
        if (ENERGY) u += e;
    }
}

// Pair (i, j): displacement from the (hi, lo) records -- the hi difference of
// two nearby floats is exact or correctly rounded relative to the result, so
// r_ij keeps ~1e-7 relative accuracy even at box sides of 68 -- then the
// cutoff test and the accumulation of F_i and (optionally) U_i.
template <bool COUL, bool ENERGY>
__device__ __forceinline__ void accum_pair(const float4& hi, const float4& lo, const float4& hj,
                                          const float4& lj, const StepArgs& a, float& fx,
                                          float& fy, float& fz, float& ue) {
    float dx = (hi.x - hj.x) + (lo.x - lj.x);
    float dy = (hi.y - hj.y) + (lo.y - lj.y);
    float dz = (hi.z - hj.z) + (lo.z - lj.z);
    float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < a.rc2) {
        float fmag, u = 0.f;
        pair_lj_coul<COUL, ENERGY>(r2, hi.w * hj.w, a, fmag, u);
        fx += fmag * dx;
        fy += fmag * dy;
        fz += fmag * dz;
        if (ENERGY) ue += u;
    }
}

// One thread per atom.  MODE 0: step (force, pending half kick, kick, drift,
// reflect, new shadow).  MODE 1: measure (force, integer-step velocity and
// energies; state untouched).
template <bool COUL, bool MASS, bool FIRST, int MODE>
__global__ void __launch_bounds__(128) k_md_step(StepArgs a) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < a.n;
    if (MODE == 0 && !valid) return;
    if (!valid) i = a.n - 1;  // measure: idle lanes join the warp reduction with zeros
    const float4 hi = __ldg(&a.sh_in[2 * (int64_t)i]);
    const float4 lo = __ldg(&a.sh_in[2 * (int64_t)i + 1]);
    const int32_t cnt = valid ? __ldg(&a.ncount[i]) : 0;
    float fx = 0.f, fy = 0.f, fz = 0.f, ue = 0.f;
    const int32_t* __restrict__ nb = a.nbr + i;
    const int64_t stride = a.n;
    // Neighbours in groups of four: the four index loads and eight record
    // loads of a group are independent, so they are in flight together.
    int32_t s = 0;
    for (; s + 4 <= cnt; s += 4) {
        int32_t j[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) j[k] = __ldg(nb + (int64_t)(s + k) * stride);
        float4 hj[4], lj[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            hj[k] = __ldg(&a.sh_in[2 * (int64_t)j[k]]);
            lj[k] = __ldg(&a.sh_in[2 * (int64_t)j[k] + 1]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            accum_pair<COUL, MODE == 1>(hi, lo, hj[k], lj[k], a, fx, fy, fz, ue);
    }
    for (; s < cnt; ++s) {
        int32_t j = __ldg(nb + (int64_t)s * stride);
        float4 hj = __ldg(&a.sh_in[2 * (int64_t)j]);
        float4 lj = __ldg(&a.sh_in[2 * (int64_t)j + 1]);
        accum_pair<COUL, MODE == 1>(hi, lo, hj, lj, a, fx, fy, fz, ue);
    }
    if (valid) a.f_out[i] = make_float4(fx, fy, fz, 0.f);
    const double imv = MASS ? a.im[i] : 1.0;
    const float fv[3] = {fx, fy, fz};
    if (MODE == 1) {
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
        // warp reduction then one FP64 atomic per warp (all 32 lanes present)
        for (int s = 16; s > 0; s >>= 1) {
            pe += __shfl_xor_sync(0xffffffffu, pe, s);
            ke += __shfl_xor_sync(0xffffffffu, ke, s);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&a.acc[0], pe);
            atomicAdd(&a.acc[1], ke);
        }
        return;
    }
    float h[3], l[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double kick = (double)(a.hdt * fv[d]) * imv;
        double v = FIRST ? a.w[d][i] : a.w[d][i] + kick;  // completes v_n
        v = v + kick;                                      // v_{n+1/2}
        double x = fma(a.dt, v, a.x[d][i]);                // x_{n+1}
        if (a.lo[d] > x) { v = -v; x = a.lo[d]; }          // boundary_reflect!
        if (a.hi[d] < x) { v = -v; x = a.hi[d]; }
        a.x[d][i] = x;
        a.w[d][i] = v;
        split_df(x, h[d], l[d]);
    }
    a.sh_out[2 * (int64_t)i] = make_float4(h[0], h[1], h[2], hi.w);
    a.sh_out[2 * (int64_t)i + 1] = make_float4(l[0], l[1], l[2], 0.f);
    // A list built at r_c + skin stays valid while no atom moved more than
    // skin/2 since the build; count the atom-steps that broke that bound.
    const float4 pb = __ldg(&a.pos_build[i]);
    const float ex = h[0] - pb.x, ey = h[1] - pb.y, ez = h[2] - pb.z;
    if (ex * ex + ey * ey + ez * ez > a.half_skin2) atomicAdd(a.diag, 1ull);
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

// Reference call shape: forces over an explicit (1-based) pair list.
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
        float hx, lx, hy, ly, hz, lz, gx, mx, gy, my, gz, mz;
        split_df(x[3 * (int64_t)i], hx, lx); split_df(x[3 * (int64_t)i + 1], hy, ly);
        split_df(x[3 * (int64_t)i + 2], hz, lz);
        split_df(x[3 * (int64_t)j], gx, mx); split_df(x[3 * (int64_t)j + 1], gy, my);
        split_df(x[3 * (int64_t)j + 2], gz, mz);
        float dx = (hx - gx) + (lx - mx), dy = (hy - gy) + (ly - my), dz = (hz - gz) + (lz - mz);
        float r2 = dx * dx + dy * dy + dz * dz;
        if (!(r2 < rc2)) continue;
        StepArgs a;
        a.sig2 = sig2; a.eps24 = eps24; a.eps4 = eps4; a.kc = kc;
        float fmag, u = 0.f;
        float qq = q ? (float)q[i] * (float)q[j] : 0.f;
        if (q) pair_lj_coul<true, true>(r2, qq, a, fmag, u);
        else pair_lj_coul<false, true>(r2, qq, a, fmag, u);
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
    int32_t n = 0, nL = 0, apl = 4, cap = 0;
    bool has_q = false, has_m = false;
    bool first = true;
    int cur = 0;        // current state set
    int sh = 0;         // current shadow buffer
    int32_t in_window = 0;  // steps done in the current window
    bool rebuild_due = false;
    int64_t steps = 0, rebuilds = 0;
    DevBuf set_buf[2], sh_buf[2], xyz32, pos32, keys, store, nbr, ncount, f, vtmp, acc, aos, diag;
    SetPtrs set[2];
    float4* shadow[2];
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int64_t graph_launches = 0;  // kernels per captured window
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
        if ((st = ensure(c, m->sh_buf[s], 2 * n * sizeof(float4)))) return st;
        m->shadow[s] = (float4*)m->sh_buf[s].p;
    }
    if ((st = ensure(c, m->xyz32, 3 * n * sizeof(float)))) return st;
    if ((st = ensure(c, m->pos32, n * sizeof(float4)))) return st;
    if ((st = ensure(c, m->keys, 32 * (size_t)(2 * m->nL)))) return st;
    if ((st = ensure(c, m->store, sizeof(int32_t) * (size_t)m->nL))) return st;
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

static StepArgs md_step_args(MDEngine* m, int shadow_in) {
    StepArgs a{};
    const nd_md_params& p = m->p;
    a.n = m->n;
    a.nbr = (const int32_t*)m->nbr.p;
    a.ncount = (const int32_t*)m->ncount.p;
    a.sh_in = m->shadow[shadow_in];
    a.sh_out = m->shadow[shadow_in ^ 1];
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
    a.pos_build = (const float4*)m->pos32.p;
    a.diag = (unsigned long long*)m->diag.p;
    {
        float hs = (float)(0.5 * p.skin);
        a.half_skin2 = hs * hs;
    }
    a.rc2 = (float)(p.cutoff * p.cutoff);
    a.sig2 = (float)(p.sigma * p.sigma);
    a.eps24 = (float)(24.0 * p.epsilon);
    a.eps4 = (float)(4.0 * p.epsilon);
    a.kc = (float)p.coulomb_k;
    a.hdt = (float)(0.5 * p.dt);
    a.dt = p.dt;
    return a;
}

template <int MODE>
static void launch_step(MDEngine* m, const StepArgs& a, bool first) {
    Ctx* c = &m->sub;
    const unsigned grid = (unsigned)cdiv(m->n, 128);
    const bool coul = m->has_q && m->p.coulomb_k != 0.0;
    const bool mass = m->has_m;
#define ND_STEP(C, M, F) k_md_step<C, M, F, MODE><<<grid, 128, 0, c->stream>>>(a)
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
// build -> full neighbour list.  Switches the current state set.
static nd_status md_rebuild(MDEngine* m) {
    Ctx* c = &m->sub;
    const int32_t n = m->n;
    const unsigned g = (unsigned)cdiv(n, 256);
    SetPtrs& s = m->set[m->cur];
    SetPtrs& t = m->set[m->cur ^ 1];
    k_md_pos32<<<g, 256, 0, c->stream>>>(s.x[0], s.x[1], s.x[2], n, (float*)m->xyz32.p);
    c->launches++;
    int32_t* codes = (int32_t*)c->codes.p;
    int32_t* perm = (int32_t*)c->perm.p;
    nd_status st;
    if ((st = morton_codes(c, (const float*)m->xyz32.p, n, m->p.order, codes, perm))) return st;
    if ((st = radix_sort_pairs(c, (uint32_t*)codes, perm, n, 30))) return st;
    k_md_reorder<<<g, 256, 0, c->stream>>>(s, t, perm, (const float*)m->xyz32.p, n,
                                           (float4*)m->pos32.p, m->shadow[0]);
    c->launches++;
    float4* keys = (float4*)m->keys.p;
    const float rl = (float)(m->p.cutoff + m->p.skin);
    k_md_leaf_boxes<<<(unsigned)cdiv(m->nL, 128), 128, 0, c->stream>>>(
        (const float4*)m->pos32.p, m->nL, m->apl, rl / 2.0f, keys);
    c->launches++;
    if ((st = build_internal_nodes(c, keys, (int32_t*)m->store.p, codes, m->nL, m->apl))) return st;
    const float hq = (rl / 2.0f) * 1.0001f + 1e-6f;
    k_md_neighbors<<<(unsigned)cdiv(n, 128), 128, 0, c->stream>>>(
        keys, (const float4*)m->pos32.p, n, m->nL, m->apl, hq, rl * rl, m->cap,
        (int32_t*)m->nbr.p, (int32_t*)m->ncount.p, c->d_err);
    c->launches++;
    m->cur ^= 1;
    m->sh = 0;
    return check_launch(c, "md rebuild");
}

// Enqueue `k` steps inside the current window (no rebuild).
static void md_steps(MDEngine* m, int32_t k) {
    for (int32_t s = 0; s < k; ++s) {
        StepArgs a = md_step_args(m, m->sh);
        launch_step<0>(m, a, m->first);
        m->first = false;
        m->sh ^= 1;
    }
}

static nd_status md_capture_window(MDEngine* m, int which) {
    // Captures rebuild + R steps starting from state set `which`.
    Ctx* c = &m->sub;
    int save_cur = m->cur, save_sh = m->sh;
    bool save_first = m->first;
    int64_t save_launch = c->launches;
    m->cur = which;
    m->first = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(c, e, "begin capture");
    nd_status st = md_rebuild(m);
    if (st == ND_OK) md_steps(m, m->p.rebuild_every);
    e = cudaStreamEndCapture(c->stream, &g);
    if (st) { if (g) cudaGraphDestroy(g); return st; }
    if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
    e = cudaGraphInstantiate(&m->graph[which], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "graph instantiate");
    m->graph_launches = c->launches - save_launch;
    c->launches = save_launch;
    m->cur = save_cur;
    m->sh = save_sh;
    m->first = save_first;
    return ND_OK;
}

static nd_status md_size_list(MDEngine* m) {
    // First build with capacity 0: counts only, then size the list.
    Ctx* c = &m->sub;
    int save_cur = m->cur;
    nd_status st = md_rebuild(m);
    if (st) return st;
    int32_t h[kErrWords];
    cudaError_t e = cudaMemcpyAsync(h, c->d_err, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "size list");
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "size list");
    if (h[0] != 0 && h[0] != ND_ERR_OVERFLOW) {
        c->last_error = "device error during the first neighbour-list build";
        cudaMemsetAsync(c->d_err, 0, sizeof(int32_t) * kErrWords, c->stream);
        return h[0];
    }
    cudaMemsetAsync(c->d_err, 0, sizeof(int32_t) * kErrWords, c->stream);
    int32_t maxc = h[2];
    int32_t cap = m->p.max_neighbors > 0 ? m->p.max_neighbors
                                         : (int32_t)std::ceil(maxc * 1.35) + 16;
    cap = (cap + 3) & ~3;
    m->cap = cap;
    if ((st = ensure(c, m->nbr, sizeof(int32_t) * (size_t)cap * (size_t)m->n))) return st;
    // The sizing build reordered the state; undo nothing (the order is free),
    // just rebuild for real with the list allocated.
    (void)save_cur;
    st = md_rebuild(m);
    if (st) return st;
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
// capacity.  ND_ERR_OVERFLOW means the caller must create a new engine.
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

static nd_status md_create_common(Ctx* parent, const nd_md_params* p, int32_t n,
                                  const double* xd, const double* vd, const double* qd,
                                  const double* md_, bool host, bool capture, MDEngine** out) {
    if (!parent || !p || !out || !xd || !vd || n <= 0) return ND_ERR_ARG;
    if (p->atomsperleaf <= 0 || n % p->atomsperleaf || n / p->atomsperleaf < 2) return ND_ERR_SPEC;
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
    m->has_q = qd != nullptr;
    m->has_m = md_ != nullptr;
    nd_status st = md_alloc(m);
    if (st) { parent->last_error = m->sub.last_error; md_destroy(m); return st; }
    Ctx* c = &m->sub;
    if ((st = md_upload(m, xd, vd, qd, md_, host))) { parent->last_error = c->last_error; md_destroy(m); return st; }
    m->cur = 0;
    m->first = true;
    if ((st = md_size_list(m))) { parent->last_error = c->last_error; md_destroy(m); return st; }
    for (int w = 0; capture && w < 2; ++w)
        if ((st = md_capture_window(m, w))) { parent->last_error = c->last_error; md_destroy(m); return st; }
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
    for (int w = 0; w < 2; ++w)
        if (m->graph[w]) cudaGraphExecDestroy(m->graph[w]);
    DevBuf* bufs[] = {&m->set_buf[0], &m->set_buf[1], &m->sh_buf[0], &m->sh_buf[1], &m->xyz32,
                      &m->pos32, &m->keys, &m->store, &m->nbr, &m->ncount, &m->f, &m->vtmp,
                      &m->acc, &m->aos, &m->diag, &m->sub.codes, &m->sub.codes_alt, &m->sub.perm,
                      &m->sub.perm_alt, &m->sub.hist, &m->sub.misc};
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
            if (steps >= R && !m->first && m->graph[m->cur]) {
                cudaError_t e = cudaGraphLaunch(m->graph[m->cur], c->stream);
                if (e != cudaSuccess) return cuda_fail(c, e, "graph launch");
                c->launches += m->graph_launches;
                m->cur ^= 1;
                m->sh = R & 1;
                m->rebuilds++;
                m->steps += R;
                steps -= R;
                continue;
            }
            if ((st = md_rebuild(m))) return st;
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
    StepArgs a = md_step_args(m, m->sh);
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
    if (capacity) *capacity = m->cap;
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
    unsigned long long v = 0;
    int32_t h[kErrWords];
    cudaError_t e = cudaMemcpyAsync(&v, m->diag.p, sizeof(v), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h, c->d_err, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "md diagnostics");
    if (skin_violations) *skin_violations = (int64_t)v;
    if (max_neighbors) *max_neighbors = h[2];
    return ND_OK;
}

int64_t md_launches_per_run(MDEngine* m, int64_t steps) {
    const int64_t R = m->p.rebuild_every;
    return (steps / R) * m->graph_launches + (steps % R) * 1;
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
