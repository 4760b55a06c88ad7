// Bug-compatible forms of the reference's force calls (src/Forces.jl), for
// scripts written against their actual results rather than the intended
// physics that the engine computes:
//
//   force_lennardjones!(force, pairslist, position)   Forces.jl:6-45
//     force zeroed; for each pair (i, j, d) in list order
//       force[i] .+= (24 eps / d) * ((2 sigma / d)^12 - (sigma / d)^6)
//     with eps = -1f10 (Float32) and sigma = 0.0001 (Float64) hard-coded, the
//     scalar added to all three components, nothing added to force[j];
//   force_coulomb!(force, pairslist, charge)           Forces.jl:46-66
//     force zeroed; for each pair in list order
//       force[i] .+= k q_i q_j / d^2  (k = 1);  force[j] .-= force[i]
//     -- the running total of force[i], an order-dependent recurrence.
//
// Precision follows Julia's promotion rules: Float32 pair distance and
// charges, 24 eps / d in Float32, the powers of sigma / d in Float64 (sigma is
// a Float64 literal), their product with the Float32 factor in Float64, added
// to the Float32 accumulator in Float64 and rounded back to Float32.  Julia's
// x^n for Float64 x and integer-valued exponent is the compensated power by
// squaring of Base.Math (pow_body), restated in jl_pow_int.
//
//   simulate!(sys, spec, clct)                         Simulator.jl:154-256
//     over the all-pairs list, Float32 state, integer stepwidth (compat_simulate).
//
// LJ: each atom's additions are independent of other atoms' -- the pairs are
// sorted by i (stable, so each atom keeps its list order) and one thread per
// atom adds its run.  Coulomb: every update reads the result of earlier ones
// through force[i] and force[j]; for an arbitrary list the recurrence runs on
// one thread in list order, for the all-pairs order of unique_pairs it splits
// into levels of independent pairs (compat_simulate).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "nd_internal.cuh"

namespace nd {

namespace {

// Julia's Base.Math.pow_body(x::Float64, n::Integer) for n >= 4: power by
// squaring with the low parts of each product kept (two_mul) and folded in
// with fused multiply-adds (Julia's muladd, fused on the hosts the reference
// targets).  Every other operation is rounded on its own (__d*_rn: nothing is
// contracted).
__device__ inline double jl_pow_int(double x, int n) {
    double y = 1.0, xnlo = 0.0, ynlo = 0.0;
    while (n > 1) {
        if (n & 1) {
            const double err = fma(y, xnlo, __dmul_rn(x, ynlo));
            const double yy = __dmul_rn(x, y);
            ynlo = __dadd_rn(fma(x, y, -yy), err);
            y = yy;
        }
        const double err = __dmul_rn(__dmul_rn(x, 2.0), xnlo);
        const double xx = __dmul_rn(x, x);
        xnlo = __dadd_rn(fma(x, x, -xx), err);
        x = xx;
        n >>= 1;
    }
    const double err = fma(y, xnlo, __dmul_rn(x, ynlo));
    return (isfinite(x) && isfinite(err)) ? fma(x, y, err) : __dmul_rn(x, y);
}

// lennardjones_interior (Forces.jl:6-13) for one pair distance d: the value
// added to each component of force[i].
__device__ inline double lj_compat_term(float d) {
    const float eps = -1e10f;
    const double sigma = 0.0001;
    const float a = __fdiv_rn(__fmul_rn(24.0f, eps), d);  // 24 * eps: Int times Float32
    const double b = jl_pow_int(__ddiv_rn(__dmul_rn(2.0, sigma), (double)d), 12);
    const double c = jl_pow_int(__ddiv_rn(sigma, (double)d), 6);
    return __dmul_rn((double)a, __dsub_rn(b, c));
}

__global__ void k_compat_runs(const uint32_t* __restrict__ key, int64_t np, int32_t* start,
                              int32_t* end) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const uint32_t k = key[p];  // 1-based atom index
    if (p == 0 || key[p - 1] != k) start[k - 1] = (int32_t)p;
    if (p == np - 1 || key[p + 1] != k) end[k - 1] = (int32_t)p + 1;
}

__global__ void k_compat_lj(const int32_t* __restrict__ order, const float* __restrict__ pd,
                            const int32_t* __restrict__ start, const int32_t* __restrict__ end,
                            int32_t n, float* __restrict__ force) {
    const int32_t a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    float f = 0.0f;
    for (int32_t p = start[a]; p < end[a]; ++p)
        f = (float)__dadd_rn((double)f, lj_compat_term(__ldg(&pd[__ldg(&order[p])])));
    force[3 * (int64_t)a] = f;
    force[3 * (int64_t)a + 1] = f;
    force[3 * (int64_t)a + 2] = f;
}

__global__ void k_compat_coulomb(const int32_t* __restrict__ pi, const int32_t* __restrict__ pj,
                                 const float* __restrict__ pd, int64_t np,
                                 const float* __restrict__ q, float* F, int32_t n,
                                 int32_t* err) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int64_t p = 0; p < np; ++p) {
        const int32_t i = pi[p] - 1, j = pj[p] - 1;
        if (i < 0 || i >= n || j < 0 || j >= n) { set_error(err, ND_ERR_ARG, (int32_t)p); return; }
        const float d = pd[p];
        // k * charge[i] * charge[j] ./ (d .^ 2), k = 1
        F[i] = __fadd_rn(F[i], __fdiv_rn(__fmul_rn(q[i], q[j]), __fmul_rn(d, d)));
        F[j] = __fsub_rn(F[j], F[i]);
    }
}

__global__ void k_compat_spread(const float* __restrict__ F, int32_t n, float* __restrict__ force) {
    const int32_t a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const float f = F[a];
    force[3 * (int64_t)a] = f;
    force[3 * (int64_t)a + 1] = f;
    force[3 * (int64_t)a + 2] = f;
}

__global__ void k_iota(int32_t* v, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) v[p] = (int32_t)p;
}

// ------------------------------------------------ simulate! as written
// The all-pairs list of unique_pairs (AllToAll.jl:65-80) holds (i, j) for
// i < j, row by row (row i: j = i + 1 .. n - 1, 0-based).  Nothing of it is
// stored in that order: the Lennard-Jones terms are stored by offset
// k = j - i - 1 along the rows (entry (k, i) at koff(k) + i, so the threads
// of consecutive atoms read consecutive entries), the Coulomb terms by level.

__host__ __device__ inline int64_t koff(int32_t k, int32_t n) {
    return (int64_t)k * (n - 1) - (int64_t)k * (k - 1) / 2;
}

// update_pairslist! (AllToAll.jl:7-62): d = sqrt(sum((a[i] .- a[j]).^2)),
// the sum left to right, and the pair's force_lennardjones! term
// (lennardjones_interior depends on d alone) with whether d < thr
// (threshold_pairs, AllToAll.jl:83-88).  One block per row.
__global__ void k_cs_pairs(const float* __restrict__ x, int32_t n, float thr,
                           double* __restrict__ ljt, unsigned char* __restrict__ near) {
    const int32_t i = blockIdx.x;
    const float xi = x[3 * (int64_t)i], yi = x[3 * (int64_t)i + 1], zi = x[3 * (int64_t)i + 2];
    for (int32_t j = i + 1 + threadIdx.x; j < n; j += blockDim.x) {
        const float dx = __fsub_rn(xi, x[3 * (int64_t)j]);
        const float dy = __fsub_rn(yi, x[3 * (int64_t)j + 1]);
        const float dz = __fsub_rn(zi, x[3 * (int64_t)j + 2]);
        const float dd = __fsqrt_rn(
            __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
        const int64_t e = koff(j - i - 1, n) + i;
        ljt[e] = lj_compat_term(dd);
        near[e] = dd < thr;
    }
}

// force_lennardjones! over the whole list and over threshold_pairs(list,
// thr): atom i's terms are its row, added in order to Float32 accumulators,
// each addition rounded through Float64 as Julia's promotion does.  One thread
// per atom, one warp per block so that the atoms' serial Float64 additions
// spread over the SMs' Float64 pipes; the loads run 16 terms ahead.
__global__ void k_cs_lj(const double* __restrict__ ljt, const unsigned char* __restrict__ near,
                        int32_t n, float* __restrict__ ljthr, float* __restrict__ ljall) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t L = n - 1 - i;
    float fa = 0.0f, ft = 0.0f;
    int64_t e = i;  // koff(0) + i
    int32_t k = 0;
    for (; k + 16 <= L; k += 16) {
        double t[16];
        unsigned char u[16];
        int64_t ee = e;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            t[r] = __ldg(&ljt[ee]);
            u[r] = __ldg(&near[ee]);
            ee += n - 1 - (k + r);
        }
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            fa = __double2float_rn(__dadd_rn((double)fa, t[r]));
            if (u[r]) ft = __double2float_rn(__dadd_rn((double)ft, t[r]));
        }
        e = ee;
    }
    for (; k < L; ++k) {
        const double t = __ldg(&ljt[e]);
        fa = __double2float_rn(__dadd_rn((double)fa, t));
        if (__ldg(&near[e])) ft = __double2float_rn(__dadd_rn((double)ft, t));
        e += n - 1 - k;
    }
    ljthr[i] = ft;
    ljall[i] = fa;
}

// force_coulomb! over the all-pairs list.  Pair (i, j) depends on the pairs
// before it that touch i or j: in this list order those are (i, j - 1) (or
// (i - 1, i)) and (i - 1, j), so the pairs with i + j = s form one level
// whose pairs touch distinct atoms, and level s follows level s - 1.  Running
// the levels in order, each pair's two updates exactly as written, gives every
// atom the same sequence of roundings as the sequential loop.
//
// The pair terms k q_i q_j / d^2 do not depend on the recurrence: they are
// computed in parallel beforehand and stored level by level (level s at
// s * stride for the shared-memory form, at level_off(s) when packed; its
// pairs by increasing i), so each level is one contiguous, coalesced segment.

__host__ __device__ inline int32_t level_lo(int32_t s, int32_t n) { return max(0, s - (n - 1)); }
__host__ __device__ inline int32_t level_count(int32_t s, int32_t n) {
    return (s - 1) / 2 - level_lo(s, n) + 1;
}
// Pairs in the levels before s: level t <= n - 1 holds ceil(t / 2) pairs, so
// floor(s^2 / 4) for s <= n; the map (i, j) -> (n-1-j, n-1-i) reverses the
// levels, which gives P - floor((2n - 1 - s)^2 / 4) for s >= n - 1.
__host__ __device__ inline int64_t level_off(int32_t s, int32_t n) {
    if (s <= n) return (int64_t)s * s / 4;
    const int64_t r = 2 * (int64_t)n - 1 - s;
    return (int64_t)n * (n - 1) / 2 - r * r / 4;
}

// The pair terms of one level per block, from the positions with the same
// operations as update_pairslist! (so the same d).
// stride > 0: level s at s * stride (16-byte aligned segments); else packed.
__global__ void k_cs_cterms(const float* __restrict__ x, const float* __restrict__ q, int32_t n,
                            int32_t stride, float* __restrict__ cterm) {
    const int32_t s = blockIdx.x + 1;
    const int32_t ilo = level_lo(s, n), cnt = level_count(s, n);
    float* out = cterm + (stride ? (int64_t)s * stride : level_off(s, n));
    for (int32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
        const int32_t i = ilo + k, j = s - i;
        const float dx = __fsub_rn(x[3 * (int64_t)i], x[3 * (int64_t)j]);
        const float dy = __fsub_rn(x[3 * (int64_t)i + 1], x[3 * (int64_t)j + 1]);
        const float dz = __fsub_rn(x[3 * (int64_t)i + 2], x[3 * (int64_t)j + 2]);
        const float d = __fsqrt_rn(
            __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
        // k * charge[i] * charge[j] ./ (d .^ 2), k = 1
        out[k] = __fdiv_rn(__fmul_rn(q[i], q[j]), __fmul_rn(d, d));
    }
}

__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(src) : "memory");
}

constexpr int kRingThreads = 128;  // fewest warps paying the per-level overhead (measured: 128 of 32-1024)
constexpr int kLevelBatch = 8;  // pairs of a level per thread with their loads in flight

// The recurrence, accumulators in shared memory, the pair terms of the next
// RING - 1 levels copied ahead into a shared ring in 16-byte pieces (levels
// at a fixed 16-byte-aligned stride).  One barrier per level: after a level's
// updates each thread waits for its own copies of the next level, and the
// barrier makes every thread's updates and copies visible to all.
template <int RING>
__global__ void __launch_bounds__(kRingThreads, 1) k_cs_coulomb_ring(const float* __restrict__ cterm,
                                                                     int32_t n, int32_t stride,
                                                                     float* __restrict__ F) {
    extern __shared__ float4 sh4[];
    float* ring = reinterpret_cast<float*>(sh4);  // RING x stride, 16-byte aligned
    float* f = ring + (int64_t)RING * stride;
    for (int32_t k = threadIdx.x; k < n; k += blockDim.x) f[k] = 0.0f;
    const int32_t smax = 2 * n - 3;
    auto issue = [&](int32_t s) {
        if (s <= smax) {
            const int32_t pieces = (level_count(s, n) + 3) >> 2;
            const float* src = cterm + (int64_t)s * stride;
            float* dst = ring + (s % RING) * (int64_t)stride;
            for (int32_t k = threadIdx.x; k < pieces; k += blockDim.x)
                cp_async16(dst + 4 * k, src + 4 * k);
        }
        cp_async_commit();  // one group per level, empty or not
    };
    for (int32_t s = 1; s < RING; ++s) issue(s);
    cp_async_wait<RING - 2>();  // level 1
    __syncthreads();
    for (int32_t s = 1; s <= smax; ++s) {
        const float* cc = ring + (s % RING) * (int64_t)stride;
        const int32_t ilo = level_lo(s, n), ihi = (s - 1) / 2;
        // the pairs of a level touch distinct atoms: all of this thread's
        // loads go first, then the updates (kLevelBatch pairs at a time)
        for (int32_t i0 = ilo + (int32_t)threadIdx.x; i0 <= ihi;
             i0 += kLevelBatch * (int32_t)blockDim.x) {
            float a[kLevelBatch], b[kLevelBatch], t[kLevelBatch];
#pragma unroll
            for (int m = 0; m < kLevelBatch; ++m) {
                const int32_t i = i0 + m * (int32_t)blockDim.x;
                if (i <= ihi) {
                    a[m] = f[i];
                    b[m] = f[s - i];
                    t[m] = cc[i - ilo];
                }
            }
#pragma unroll
            for (int m = 0; m < kLevelBatch; ++m) {
                const int32_t i = i0 + m * (int32_t)blockDim.x;
                if (i <= ihi) {
                    const float fi = __fadd_rn(a[m], t[m]);
                    f[i] = fi;
                    f[s - i] = __fsub_rn(b[m], fi);
                }
            }
        }
        issue(s + RING - 1);
        cp_async_wait<RING - 2>();  // this thread's pieces of level s + 1
        __syncthreads();
    }
    cp_async_wait<0>();
    for (int32_t k = threadIdx.x; k < n; k += blockDim.x) F[k] = f[k];
}

// The same recurrence with the accumulators in global memory (any n): the
// block's own writes are visible to it after each barrier.  The first item of
// the next level is loaded ahead.
__global__ void __launch_bounds__(kRingThreads, 1) k_cs_coulomb_global(const float* __restrict__ cterm,
                                                               int32_t n, float* F) {
    for (int32_t k = threadIdx.x; k < n; k += blockDim.x) F[k] = 0.0f;
    __syncthreads();
    const int32_t smax = 2 * n - 3;
    auto first = [&](int32_t s) -> float {
        if (s > smax || (int32_t)threadIdx.x >= level_count(s, n)) return 0.0f;
        return __ldg(&cterm[level_off(s, n) + threadIdx.x]);
    };
    float cn = first(1);
    for (int32_t s = 1; s <= smax; ++s) {
        const float c0 = cn;
        cn = first(s + 1);
        const int32_t ilo = level_lo(s, n), ihi = (s - 1) / 2;
        const float* cc = cterm + level_off(s, n);
        for (int32_t i = ilo + (int32_t)threadIdx.x; i <= ihi; i += blockDim.x) {
            const int32_t j = s - i;
            const float c = i == ilo + (int32_t)threadIdx.x ? c0 : __ldg(&cc[i - ilo]);
            const float fi = __fadd_rn(F[i], c);
            F[i] = fi;
            F[j] = __fsub_rn(F[j], fi);
        }
        __syncthreads();
    }
}

// One step's per-atom part (Simulator.jl:183-228): sum_forces!, the position
// update with a(t), the velocity update with a(t) + a(t - dt) (Fnext, the
// previous step's all-pairs forces), boundary_reflect! (:81-111), and the
// forces carried to the next step.  Every operation rounds to Float32 as in
// Julia (Float32 times Int64 promotes to Float32).
__global__ void k_cs_step(float* __restrict__ x, float* __restrict__ v, float* __restrict__ force,
                          float* __restrict__ fnext, const float* __restrict__ mass,
                          const float* __restrict__ ljthr, const float* __restrict__ ljall,
                          const float* __restrict__ cf, int32_t n, float dt, float dt2,
                          float3 lo, float3 hi, float* __restrict__ frame) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float m = mass[i];
    const float at = __fdiv_rn(__fadd_rn(ljthr[i], cf[i]), m);  // accels_t
    const float fn = __fadd_rn(ljall[i], cf[i]);                // force_nextstep
    const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int64_t e = 3 * (int64_t)i + k;
        float xk = x[e], vk = v[e];
        // position .+= velocity .* dt .+ ((accels_t .* dt ^ 2) ./ 2)
        xk = __fadd_rn(xk, __fadd_rn(__fmul_rn(vk, dt), __fdiv_rn(__fmul_rn(at, dt2), 2.0f)));
        const float atdt = __fdiv_rn(fnext[e], m);  // accels_t_dt
        // velocity .+= (accels_t .+ accels_t_dt) .* dt / 2
        vk = __fadd_rn(vk, __fdiv_rn(__fmul_rn(__fadd_rn(at, atdt), dt), 2.0f));
        if (l[k] > xk) {
            vk = __fmul_rn(vk, -1.0f);
            xk = l[k];
        }
        if (h[k] < xk) {
            vk = __fmul_rn(vk, -1.0f);
            xk = h[k];
        }
        x[e] = xk;
        v[e] = vk;
        force[e] = fn;
        fnext[e] = fn;
        if (frame) frame[e] = xk;
    }
}

// rescale_velocity!(velocity, Tf, gamma, mass, objectcount) (Simulator.jl:
// 119-144): Ti += (2 / (3 objects kb)) * |v_i| * m_i / 2 in Float32, in atom
// order; beta = (1 + gamma (Tf / Ti - 1))^0.5 in Float64 (Float32 ^ Float64
// promotes; the square root correctly rounded); v .*= beta through Float64.
// A negative radicand raises ND_ERR_ARG and leaves v unchanged.  One block.
__global__ void __launch_bounds__(1024) k_cs_rescale(float* __restrict__ v,
                                                     const float* __restrict__ mass, int32_t n,
                                                     float c, float Tf, float gamma,
                                                     float* __restrict__ term, int32_t* err) {
    __shared__ double beta;
    __shared__ int ok;
    for (int32_t k = threadIdx.x; k < n; k += blockDim.x) {
        const float a = v[3 * (int64_t)k], b = v[3 * (int64_t)k + 1], z = v[3 * (int64_t)k + 2];
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(z, z));
        term[k] = __fdiv_rn(__fmul_rn(__fmul_rn(c, __fsqrt_rn(s)), mass[k]), 2.0f);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float Ti = 0.0f;
        for (int32_t k = 0; k < n; ++k) Ti = __fadd_rn(Ti, term[k]);
        const float r = __fadd_rn(1.0f, __fmul_rn(gamma, __fsub_rn(__fdiv_rn(Tf, Ti), 1.0f)));
        ok = !(r < 0.0f);
        if (ok) beta = __dsqrt_rn((double)r);
        else set_error(err, ND_ERR_ARG, 1);
    }
    __syncthreads();
    if (!ok) return;
    for (int64_t e = threadIdx.x; e < 3 * (int64_t)n; e += blockDim.x)
        v[e] = __double2float_rn(__dmul_rn((double)v[e], beta));
}

}  // namespace

nd_status compat_simulate(Ctx* c, const nd_compat_sim* spec, int32_t n, float* x, float* v,
                          float* force, const float* mass, const float* q, float* poslog) {
    if (!spec || !x || !v || !force || !mass || !q) return ND_ERR_ARG;
    if (n < 1 || n > 65536 || spec->duration < 0) {
        c->last_error = "nd_compat_simulate: 1 <= n <= 65536 and duration >= 0";
        return ND_ERR_ARG;
    }
    const size_t n3 = 3 * (size_t)n;
    const int64_t P = (int64_t)n * (n - 1) / 2;
    // device log: a chunk of frames, flushed to the host when full
    const int64_t frame_bytes = (int64_t)(n3 * sizeof(float));
    int64_t chunk_frames = (256ll << 20) / frame_bytes;
    // test hooks: a smaller log chunk (several flushes) and the global-memory
    // Coulomb form at any size; both compute the same results
    if (const char* ev = getenv("NAIVEGPU_COMPAT_LOG_CHUNK")) chunk_frames = atoll(ev);
    const bool force_global = getenv("NAIVEGPU_COMPAT_GLOBAL") != nullptr;
    const int64_t chunk =
        poslog ? std::max<int64_t>(1, std::min<int64_t>(spec->duration, chunk_frames)) : 0;
    nd_status st;
    // Coulomb terms: levels at a 16-byte-aligned stride when the recurrence
    // runs in shared memory (the widest level is level n - 1), else packed
    const int32_t maxc = n > 1 ? level_count(n - 1, n) : 1;
    const int32_t stride = (maxc + 3) & ~3;
    auto shmem = [&](int r) { return sizeof(float) * ((size_t)r * stride + (size_t)n); };
    int ring = 0;
    for (int r : {8, 4, 3})
        if (!ring && !force_global && shmem(r) <= 200 * 1024) ring = r;
    const int32_t nlev = std::max(2 * n - 3, 0);
    const size_t ncterm = ring ? (size_t)(nlev + 1) * stride : (size_t)std::max<int64_t>(P, 1);
    if ((st = ensure(c, c->leafpairs, sizeof(float) * ncterm))) return st;
    if ((st = ensure(c, c->pairs_i, sizeof(double) * (size_t)std::max<int64_t>(P, 1)))) return st;
    if ((st = ensure(c, c->pairs_j, (size_t)std::max<int64_t>(P, 1)))) return st;
    const size_t small = sizeof(float) * (4 * n3 + 6 * (size_t)n);
    if ((st = ensure(c, c->compat, small + (size_t)(chunk * frame_bytes)))) return st;
    float* cterm = (float*)c->leafpairs.p;               // Coulomb pair terms, by level
    double* ljt = (double*)c->pairs_i.p;                 // LJ pair terms, by row offset
    unsigned char* near = (unsigned char*)c->pairs_j.p;  // d < 0.01, same layout
    float* dx = (float*)c->compat.p;
    float* dv = dx + n3;
    float* dF = dv + n3;
    float* dFn = dF + n3;
    float* dm = dFn + n3;
    float* dq = dm + n;
    float* ljthr = dq + n;
    float* ljall = ljthr + n;
    float* cf = ljall + n;
    float* term = cf + n;
    float* dlog = term + n;
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemcpyAsync(dx, x, n3 * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dv, v, n3 * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)  // force_nextstep = deepcopy(sys.force)
        e = cudaMemcpyAsync(dFn, force, n3 * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dF, force, n3 * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dm, mass, n * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dq, q, n * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "compat simulate upload");

    const size_t shb = ring ? shmem(ring) : 0;
    if (ring) {
        const void* fn = ring == 8   ? (const void*)k_cs_coulomb_ring<8>
                         : ring == 4 ? (const void*)k_cs_coulomb_ring<4>
                                     : (const void*)k_cs_coulomb_ring<3>;
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shb);
        if (e != cudaSuccess) return cuda_fail(c, e, "compat simulate smem");
    }
    // Two chains per step, both from the list of the previous step's
    // positions: force_coulomb! (update_pairslist!'s Coulomb terms, then the
    // levels on one SM) on the context's stream, and force_lennardjones!
    // (the LJ terms of update_pairslist!, then the row sums) on a side stream
    // over the other SMs.  The step kernel waits for both; the side chain of
    // the next step waits for the step kernel.
    struct Side {
        cudaStream_t s2 = nullptr;
        cudaEvent_t moved = nullptr, lj = nullptr;
        ~Side() {
            if (s2) cudaStreamSynchronize(s2);
            if (moved) cudaEventDestroy(moved);
            if (lj) cudaEventDestroy(lj);
            if (s2) cudaStreamDestroy(s2);
        }
    } side;
    e = cudaStreamCreateWithFlags(&side.s2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&side.moved, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&side.lj, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(c, e, "compat simulate streams");
    cudaStream_t s2 = side.s2;
    auto coulomb_terms = [&]() {
        if (n > 1) {
            k_cs_cterms<<<nlev, 256, 0, s>>>(dx, dq, n, ring ? stride : 0, cterm);
            c->launches++;
        }
    };
    auto coulomb = [&]() {
        if (ring == 8)
            k_cs_coulomb_ring<8><<<1, kRingThreads, shb, s>>>(cterm, n, stride, cf);
        else if (ring == 4)
            k_cs_coulomb_ring<4><<<1, kRingThreads, shb, s>>>(cterm, n, stride, cf);
        else if (ring == 3)
            k_cs_coulomb_ring<3><<<1, kRingThreads, shb, s>>>(cterm, n, stride, cf);
        else
            k_cs_coulomb_global<<<1, kRingThreads, 0, s>>>(cterm, n, cf);
        c->launches++;
    };
    // after the positions of stream `after` moved: the LJ terms and sums on s2
    auto lj_chain = [&](cudaStream_t after) -> cudaError_t {
        cudaError_t ee = cudaEventRecord(side.moved, after);
        if (ee == cudaSuccess) ee = cudaStreamWaitEvent(s2, side.moved, 0);
        if (ee != cudaSuccess) return ee;
        if (n > 1) k_cs_pairs<<<n - 1, 256, 0, s2>>>(dx, n, 0.01f, ljt, near);
        k_cs_lj<<<(unsigned)cdiv(n, 32), 32, 0, s2>>>(ljt, near, n, ljthr, ljall);
        c->launches += n > 1 ? 2 : 1;
        return cudaEventRecord(side.lj, s2);
    };
    const float dt = (float)spec->stepwidth;
    const float dt2 = (float)(int64_t)((uint64_t)spec->stepwidth * (uint64_t)spec->stepwidth);
    const float3 lo = make_float3(spec->min_dim[0], spec->min_dim[1], spec->min_dim[2]);
    const float3 hi = make_float3(spec->max_dim[0], spec->max_dim[1], spec->max_dim[2]);
    // rescale_velocity!: 2 / (3 * objects * kb), objects = Float32(objectnumber), kb = 1
    const float cT = 2.0f / ((3.0f * (float)spec->objectnumber) * 1.0f);
    const unsigned ga = (unsigned)cdiv(n, 256);

    // pairslist = unique_pairs(position)
    coulomb_terms();
    if ((e = lj_chain(s)) != cudaSuccess) return cuda_fail(c, e, "compat simulate streams");
    int64_t pending = 0;  // frames in the device chunk not yet copied out
    int64_t first = 1;    // step of the chunk's first frame
    auto flush = [&]() -> nd_status {
        if (pending == 0) return ND_OK;
        cudaError_t ee = cudaMemcpyAsync(poslog + first * (int64_t)n3, dlog,
                                         (size_t)(pending * frame_bytes), cudaMemcpyDeviceToHost, s);
        if (ee != cudaSuccess) return cuda_fail(c, ee, "compat simulate log");
        ee = cudaStreamSynchronize(s);
        if (ee != cudaSuccess) return cuda_fail(c, ee, "compat simulate log");
        first += pending;
        pending = 0;
        return ND_OK;
    };
    for (int64_t step = 1; step <= spec->duration; ++step) {
        // force_coulomb! runs twice per step on the same list and charges: one
        // evaluation gives both results; so does force_lennardjones!'s pass
        // over the whole list and its threshold_pairs part
        coulomb();
        float* frame = poslog ? dlog + pending * (int64_t)n3 : nullptr;
        e = cudaStreamWaitEvent(s, side.lj, 0);
        if (e != cudaSuccess) return cuda_fail(c, e, "compat simulate streams");
        k_cs_step<<<ga, 256, 0, s>>>(dx, dv, dF, dFn, dm, ljthr, ljall, cf, n, dt, dt2, lo, hi,
                                      frame);
        c->launches++;
        if (step < spec->duration) {  // update_pairslist! (unused after the last step)
            coulomb_terms();
            if ((e = lj_chain(s)) != cudaSuccess) return cuda_fail(c, e, "compat simulate streams");
        }
        if (step % 10 == 0) {
            k_cs_rescale<<<1, 1024, 0, s>>>(dv, dm, n, cT, spec->temperature,
                                             spec->velocity_dampening, term, c->d_err);
            c->launches++;
            if ((st = sync_and_check(c, "compat simulate (rescale_velocity!)"))) {
                // the reference throws here: hand back the state it holds
                cudaMemcpyAsync(x, dx, n3 * sizeof(float), cudaMemcpyDeviceToHost, s);
                cudaMemcpyAsync(v, dv, n3 * sizeof(float), cudaMemcpyDeviceToHost, s);
                cudaMemcpyAsync(force, dF, n3 * sizeof(float), cudaMemcpyDeviceToHost, s);
                cudaStreamSynchronize(s);
                c->last_error = "rescale_velocity!: negative radicand (DomainError)";
                return st;
            }
        }
        if (poslog && ++pending == chunk && (st = flush())) return st;
        if ((st = check_launch(c, "compat simulate"))) return st;
    }
    if (poslog && (st = flush())) return st;
    e = cudaMemcpyAsync(x, dx, n3 * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v, dv, n3 * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(force, dF, n3 * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && poslog)  // poslog[1] is sys.position itself
        e = cudaMemcpyAsync(poslog, dx, n3 * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "compat simulate download");
    return sync_and_check(c, "compat simulate");
}

namespace {

// ------------------------------------------------ collect_objects
// collect_objects(::GenericRandomCollector) (MDInput.jl:305-369) with a
// counter-based stream in place of Julia's global RNG: draw k of stream c is
// mix64(seed ^ mix64(c << 56 ^ k)).  Uniform(a, b) as Distributions draws it:
// a + (b - a) * u with u in [0, 1) (53 bits), stored as Float32; rand(Float32)
// for the velocity split: 24 bits.

__host__ __device__ inline uint64_t cobj_bits(uint64_t seed, uint64_t stream, uint64_t k) {
    return mix64(seed ^ mix64((stream << 56) ^ k));
}
__host__ __device__ inline float cobj_uniform(uint64_t seed, uint64_t stream, uint64_t k, float a,
                                              float b) {
    const double u = (double)(cobj_bits(seed, stream, k) >> 11) * 0x1.0p-53;
    return (float)((double)a + (double)(b - a) * u);
}
__host__ __device__ inline float cobj_rand32(uint64_t seed, uint64_t stream, uint64_t k) {
    return (float)(cobj_bits(seed, stream, k) >> 40) * 0x1.0p-24f;
}

// mass, charge, position (generate_positions, MDInput.jl:175-190) and the
// velocity split draws of every atom.
__global__ void k_cobj_draw(nd_collector cl, uint64_t seed, int32_t n, float* __restrict__ x,
                            float* __restrict__ m, float* __restrict__ q,
                            float* __restrict__ vd) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    m[i] = cobj_uniform(seed, 0, i, cl.minmass, cl.maxmass);
    q[i] = cobj_uniform(seed, 1, i, cl.mincharge, cl.maxcharge);
    for (int d = 0; d < 3; ++d) {
        x[3 * (int64_t)i + d] = cobj_uniform(seed, 2 + d, i, cl.min_dim[d], cl.max_dim[d]);
        vd[(int64_t)d * n + i] = cobj_rand32(seed, 5 + d, i);
    }
}

// sum(veldist) per dimension in a fixed order: 256-element chunks reduced as
// a binary tree (stride 128, 64, .., 1), then the chunk sums in chunk order.
__global__ void __launch_bounds__(256) k_cobj_chunks(const float* __restrict__ vd, int32_t n,
                                                     int32_t nchunk, float* __restrict__ part) {
    __shared__ float t[256];
    const int d = blockIdx.y;
    const int64_t k = (int64_t)blockIdx.x * 256 + threadIdx.x;
    t[threadIdx.x] = k < n ? vd[(int64_t)d * n + k] : 0.0f;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) t[threadIdx.x] = __fadd_rn(t[threadIdx.x], t[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(int64_t)d * nchunk + blockIdx.x] = t[0];
}

__global__ void k_cobj_total(const float* __restrict__ part, int32_t nchunk, float* sum) {
    const int d = threadIdx.x;
    if (d >= 3) return;
    float s = 0.0f;
    for (int32_t c = 0; c < nchunk; ++c) s = __fadd_rn(s, part[(int64_t)d * nchunk + c]);
    sum[d] = s;
}

// velocity[i][d] = T * veldist[i] * 3 * N * kb / mass[i] with veldist ./=
// sum(veldist), or T / N * 3 * N * kb / mass[i] (kb = 1), in Float32.
__global__ void k_cobj_velocity(nd_collector cl, int32_t n, const float* __restrict__ m,
                                const float* __restrict__ vd, const float* __restrict__ sum,
                                float* __restrict__ v) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float N = (float)cl.objectnumber;
    for (int d = 0; d < 3; ++d) {
        float a;
        if (cl.randomvelocity) {
            const float vn = __fdiv_rn(vd[(int64_t)d * n + i], sum[d]);
            a = __fmul_rn(__fmul_rn(__fmul_rn(cl.temperature, vn), 3.0f), N);
        } else {
            a = __fmul_rn(__fmul_rn(__fdiv_rn(cl.temperature, N), 3.0f), N);
        }
        v[3 * (int64_t)i + d] = __fdiv_rn(__fmul_rn(a, 1.0f), m[i]);
    }
}

// unique_pairs_prune (MDInput.jl:228-259) as written: for i in 1:N-1, j in
// i+1:N-1 (the last atom is never compared), sqrt(dx^2 + dy^2 + dz^2) <
// minimumdistance fills a[i] with Inf.  A filled a[i] meets nothing after,
// and every a[j] compared is still the drawn one, so atom i is filled exactly
// when some j in (i, N-1) lies within the distance of it: one thread per i,
// the candidates staged through shared memory.
__global__ void __launch_bounds__(256) k_cobj_prune(const float* __restrict__ x, int32_t n,
                                                    float dmin, unsigned char* __restrict__ hit) {
    __shared__ float3 tile[256];
    const int32_t i = blockIdx.x * 256 + threadIdx.x;
    const int32_t jmax = n - 2;  // last compared atom, 0-based
    float3 a = make_float3(0.f, 0.f, 0.f);
    if (i < n) a = make_float3(x[3 * (int64_t)i], x[3 * (int64_t)i + 1], x[3 * (int64_t)i + 2]);
    bool found = false;
    for (int32_t j0 = blockIdx.x * 256; j0 <= jmax; j0 += 256) {
        const int32_t jl = j0 + threadIdx.x;
        if (jl <= jmax)
            tile[threadIdx.x] =
                make_float3(x[3 * (int64_t)jl], x[3 * (int64_t)jl + 1], x[3 * (int64_t)jl + 2]);
        __syncthreads();
        if (!found && i < jmax) {
            const int32_t kend = min(256, jmax - j0 + 1);
            for (int k = max(0, i + 1 - j0); k < kend; ++k) {
                const float dx = __fsub_rn(a.x, tile[k].x), dy = __fsub_rn(a.y, tile[k].y),
                            dz = __fsub_rn(a.z, tile[k].z);
                const float d = __fsqrt_rn(
                    __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
                if (d < dmin) {
                    found = true;
                    break;
                }
            }
        }
        __syncthreads();
    }
    if (i < n) hit[i] = found;
}

__global__ void k_cobj_fill(float* __restrict__ x, const unsigned char* __restrict__ hit, int32_t n,
                            unsigned long long* count) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !hit[i]) return;
    x[3 * (int64_t)i] = x[3 * (int64_t)i + 1] = x[3 * (int64_t)i + 2] = __int_as_float(0x7f800000);
    atomicAdd(count, 1ull);
}

}  // namespace

nd_status collect_objects(Ctx* c, const nd_collector* cl, uint64_t seed, float* x, float* v,
                          float* m, float* q, int64_t* pruned) {
    if (!cl || !x || !v || !m || !q) return ND_ERR_ARG;
    // the pruning compares every pair (as the reference does): 2^20 atoms
    // are 5e11 comparisons, about a second
    if (cl->objectnumber < 1 || cl->objectnumber > (1 << 20)) {
        c->last_error = "nd_collect_objects: 1 <= objectnumber <= 2^20";
        return ND_ERR_ARG;
    }
    const int32_t n = (int32_t)cl->objectnumber;
    const size_t n3 = 3 * (size_t)n;
    const int32_t nchunk = (int32_t)cdiv(n, 256);
    nd_status st;
    // [count (16 B)] [x, v, m, q, veldist, chunk sums, sums (Float32)] [hit (bytes)]
    const size_t nf = 2 * n3 + 2 * (size_t)n + n3 + 3 * (size_t)nchunk + 4;
    if ((st = ensure(c, c->compat, 16 + sizeof(float) * nf + (size_t)n))) return st;
    unsigned long long* cnt = (unsigned long long*)c->compat.p;
    float* dx = (float*)((char*)c->compat.p + 16);
    float* dv = dx + n3;
    float* dm = dv + n3;
    float* dq = dm + n;
    float* vd = dq + n;
    float* part = vd + n3;
    float* sum = part + 3 * (size_t)nchunk;
    unsigned char* hit = (unsigned char*)(sum + 4);
    cudaStream_t s = c->stream;
    const unsigned g = (unsigned)cdiv(n, 256);
    cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s);
    k_cobj_draw<<<g, 256, 0, s>>>(*cl, seed, n, dx, dm, dq, vd);
    if (cl->randomvelocity) {
        k_cobj_chunks<<<dim3((unsigned)nchunk, 3), 256, 0, s>>>(vd, n, nchunk, part);
        k_cobj_total<<<1, 32, 0, s>>>(part, nchunk, sum);
        c->launches += 2;
    }
    k_cobj_velocity<<<g, 256, 0, s>>>(*cl, n, dm, vd, sum, dv);
    k_cobj_prune<<<g, 256, 0, s>>>(dx, n, cl->minimumdistance, hit);
    k_cobj_fill<<<g, 256, 0, s>>>(dx, hit, n, cnt);
    c->launches += 4;
    if ((st = check_launch(c, "collect_objects"))) return st;
    unsigned long long h_cnt = 0;
    cudaError_t e = cudaMemcpyAsync(x, dx, n3 * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v, dv, n3 * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m, dm, n * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(q, dq, n * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "collect_objects download");
    if ((st = sync_and_check(c, "collect_objects"))) return st;
    if (pruned) *pruned = (int64_t)h_cnt;
    return ND_OK;
}

nd_status compat_forces(Ctx* c, int kind, int32_t n, const int32_t* pi, const int32_t* pj,
                        const float* pd, int64_t np, const float* q, float* force) {
    if (n <= 0 || np < 0 || !force || (np > 0 && (!pi || !pj || !pd)) || (kind == 1 && !q))
        return ND_ERR_ARG;
    if (np > INT32_MAX) return ND_ERR_ARG;
    for (int64_t p = 0; p < np; ++p)
        if (pi[p] < 1 || pi[p] > n || pj[p] < 1 || pj[p] > n) return ND_ERR_ARG;
    const size_t nx = 3 * (size_t)n;
    nd_status st;
    if ((st = ensure(c, c->pairs_i, sizeof(int32_t) * (size_t)std::max<int64_t>(np, 1)))) return st;
    if ((st = ensure(c, c->pairs_j, sizeof(int32_t) * (size_t)std::max<int64_t>(np, 1)))) return st;
    if ((st = ensure(c, c->pairs_d, sizeof(float) * (size_t)std::max<int64_t>(np, 1)))) return st;
    if ((st = ensure(c, c->counts, sizeof(float) * (nx + (size_t)n) + 2 * sizeof(int32_t) * n))) return st;
    int32_t* dpi = (int32_t*)c->pairs_i.p;
    int32_t* dpj = (int32_t*)c->pairs_j.p;
    float* dpd = (float*)c->pairs_d.p;
    float* dforce = (float*)c->counts.p;
    float* dF = dforce + nx;  // Coulomb accumulators, or LJ run starts / ends
    int32_t* start = (int32_t*)(dF + n);
    int32_t* end = start + n;
    cudaError_t e = cudaSuccess;
    if (np > 0) {
        e = cudaMemcpyAsync(dpi, pi, sizeof(int32_t) * np, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dpj, pj, sizeof(int32_t) * np, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dpd, pd, sizeof(float) * np, cudaMemcpyHostToDevice, c->stream);
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "compat forces upload");
    cudaMemsetAsync(dforce, 0, sizeof(float) * nx, c->stream);
    const unsigned ga = (unsigned)cdiv(n, 256);
    if (kind == 0 && np > 0) {
        // stable sort of the pairs by i: keys i (1-based), values the list positions
        if ((st = ensure(c, c->codes, sizeof(uint32_t) * np))) return st;
        if ((st = ensure(c, c->perm, sizeof(int32_t) * np))) return st;
        uint32_t* key = (uint32_t*)c->codes.p;
        int32_t* order = (int32_t*)c->perm.p;
        e = cudaMemcpyAsync(key, pi, sizeof(int32_t) * np, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "compat forces upload");
        k_iota<<<(unsigned)cdiv(np, 256), 256, 0, c->stream>>>(order, np);
        int bits = 1;
        while (bits < 31 && ((uint32_t)n >> bits) != 0) ++bits;
        if ((st = radix_sort_pairs(c, key, order, (int32_t)np, bits))) return st;
        cudaMemsetAsync(start, 0, sizeof(int32_t) * n, c->stream);
        cudaMemsetAsync(end, 0, sizeof(int32_t) * n, c->stream);
        k_compat_runs<<<(unsigned)cdiv(np, 256), 256, 0, c->stream>>>(key, np, start, end);
        k_compat_lj<<<ga, 256, 0, c->stream>>>(order, dpd, start, end, n, dforce);
        c->launches += 3;
    } else if (kind == 1) {
        float* dq = dF + n;  // charges after the accumulators (reuse of the run arrays)
        e = cudaMemcpyAsync(dq, q, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "compat forces upload");
        cudaMemsetAsync(dF, 0, sizeof(float) * n, c->stream);
        if (np > 0) {
            k_compat_coulomb<<<1, 32, 0, c->stream>>>(dpi, dpj, dpd, np, dq, dF, n, c->d_err);
            c->launches++;
        }
        k_compat_spread<<<ga, 256, 0, c->stream>>>(dF, n, dforce);
        c->launches++;
    }
    if ((st = check_launch(c, "compat forces"))) return st;
    e = cudaMemcpyAsync(force, dforce, sizeof(float) * nx, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "compat forces download");
    return sync_and_check(c, "compat forces");
}

}  // namespace nd
