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
// through force[i] and force[j]; the recurrence runs on one thread in list
// order (no parallel form reproduces its roundings).
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
// i < j in row-major order; only the distances are stored, row i (0-based)
// from tri_row(i).

__host__ __device__ inline int64_t tri_row(int32_t i, int32_t n) {
    return (int64_t)i * (2 * (int64_t)n - i - 1) / 2;
}

// update_pairslist! (AllToAll.jl:7-62): d = sqrt(sum((a[i] .- a[j]).^2)),
// the sum left to right.  One block per row.
__global__ void k_cs_pairs(const float* __restrict__ x, int32_t n, float* __restrict__ d) {
    const int32_t i = blockIdx.x;
    const float xi = x[3 * (int64_t)i], yi = x[3 * (int64_t)i + 1], zi = x[3 * (int64_t)i + 2];
    float* row = d + tri_row(i, n) - (i + 1);
    for (int32_t j = i + 1 + threadIdx.x; j < n; j += blockDim.x) {
        const float dx = __fsub_rn(xi, x[3 * (int64_t)j]);
        const float dy = __fsub_rn(yi, x[3 * (int64_t)j + 1]);
        const float dz = __fsub_rn(zi, x[3 * (int64_t)j + 2]);
        row[j] = __fsqrt_rn(
            __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    }
}

// force_lennardjones! over the whole list and over threshold_pairs(list, thr)
// (AllToAll.jl:83-88: the pairs with d < thr, in list order) in one pass.
// Atom i's terms are its row, in order; a warp per atom computes 32 terms at
// a time and adds them one by one (the Float32 accumulator, each addition
// rounded through Float64 as Julia's promotion does).
__global__ void __launch_bounds__(256) k_cs_lj(const float* __restrict__ d, int32_t n, float thr,
                                               float* __restrict__ ljthr,
                                               float* __restrict__ ljall) {
    const int32_t i = (int32_t)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const float* row = d + tri_row(i, n);
    const int32_t L = n - 1 - i;
    float fa = 0.0f, ft = 0.0f;
    for (int32_t b = 0; b < L; b += 32) {
        double t = 0.0;
        bool use = false;
        if (b + lane < L) {
            const float dd = __ldg(&row[b + lane]);
            t = lj_compat_term(dd);
            use = dd < thr;
        }
        const unsigned used = __ballot_sync(0xffffffffu, use);
        const int cnt = min(32, L - b);
        for (int k = 0; k < cnt; ++k) {
            const double tk = __shfl_sync(0xffffffffu, t, k);
            fa = __double2float_rn(__dadd_rn((double)fa, tk));
            if ((used >> k) & 1u) ft = __double2float_rn(__dadd_rn((double)ft, tk));
        }
    }
    if (lane == 0) {
        ljthr[i] = ft;
        ljall[i] = fa;
    }
}

// force_coulomb! over the all-pairs list.  Pair (i, j) depends on the pairs
// before it that touch i or j: in this list order those are (i, j - 1) (or
// (i - 1, i)) and (i - 1, j), so the pairs with i + j = s form one level
// whose pairs touch distinct atoms, and level s follows level s - 1.  Running
// the levels in order, each pair's two updates exactly as written, gives every
// atom the same sequence of roundings as the sequential loop.  One block;
// the accumulators (and charges) in shared memory when they fit.
template <bool SMEM>
__global__ void __launch_bounds__(1024, 1) k_cs_coulomb(const float* __restrict__ d,
                                                        const float* __restrict__ q, int32_t n,
                                                        float* __restrict__ F) {
    extern __shared__ float sh[];
    float* f = SMEM ? sh : F;
    const float* qq = SMEM ? sh + n : q;
    for (int32_t k = threadIdx.x; k < n; k += blockDim.x) {
        f[k] = 0.0f;
        if (SMEM) sh[n + k] = q[k];
    }
    __syncthreads();
    const int32_t smax = 2 * n - 3;
    // the first pair of this thread in the next level, loaded ahead
    auto first = [&](int32_t s) -> float {
        const int32_t i = max(0, s - (n - 1)) + (int32_t)threadIdx.x;
        if (s > smax || i > (s - 1) / 2) return 0.0f;
        return __ldg(&d[tri_row(i, n) + (s - 2 * i - 1)]);
    };
    float dn = first(1);
    for (int32_t s = 1; s <= smax; ++s) {
        const float dc = dn;
        dn = first(s + 1);
        const int32_t ilo = max(0, s - (n - 1)), ihi = (s - 1) / 2;
        for (int32_t i = ilo + (int32_t)threadIdx.x; i <= ihi; i += blockDim.x) {
            const int32_t j = s - i;
            const float dd = i == ilo + (int32_t)threadIdx.x ? dc
                                                             : __ldg(&d[tri_row(i, n) + (j - i - 1)]);
            // k * charge[i] * charge[j] ./ (d .^ 2), k = 1
            const float c = __fdiv_rn(__fmul_rn(qq[i], qq[j]), __fmul_rn(dd, dd));
            const float fi = __fadd_rn(f[i], c);
            f[i] = fi;
            f[j] = __fsub_rn(f[j], fi);
        }
        __syncthreads();
    }
    if (SMEM)
        for (int32_t k = threadIdx.x; k < n; k += blockDim.x) F[k] = sh[k];
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
    if ((st = ensure(c, c->pairs_d, sizeof(float) * (size_t)std::max<int64_t>(P, 1)))) return st;
    const size_t small = sizeof(float) * (4 * n3 + 6 * (size_t)n);
    if ((st = ensure(c, c->compat, small + (size_t)(chunk * frame_bytes)))) return st;
    float* dd = (float*)c->pairs_d.p;
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

    const bool smem = !force_global && 2 * (size_t)n * sizeof(float) <= 200 * 1024;
    const size_t shb = smem ? 2 * (size_t)n * sizeof(float) : 0;
    if (smem) {
        e = cudaFuncSetAttribute(k_cs_coulomb<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)shb);
        if (e != cudaSuccess) return cuda_fail(c, e, "compat simulate smem");
    }
    const float dt = (float)spec->stepwidth;
    const float dt2 = (float)(int64_t)((uint64_t)spec->stepwidth * (uint64_t)spec->stepwidth);
    const float3 lo = make_float3(spec->min_dim[0], spec->min_dim[1], spec->min_dim[2]);
    const float3 hi = make_float3(spec->max_dim[0], spec->max_dim[1], spec->max_dim[2]);
    // rescale_velocity!: 2 / (3 * objects * kb), objects = Float32(objectnumber), kb = 1
    const float cT = 2.0f / ((3.0f * (float)spec->objectnumber) * 1.0f);
    const unsigned ga = (unsigned)cdiv(n, 256);
    const unsigned gw = (unsigned)cdiv((int64_t)n * 32, 256);

    if (n > 1) {
        k_cs_pairs<<<n - 1, 256, 0, s>>>(dx, n, dd);  // pairslist = unique_pairs(position)
        c->launches++;
    }
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
        k_cs_lj<<<gw, 256, 0, s>>>(dd, n, 0.01f, ljthr, ljall);
        // force_coulomb! runs twice per step on the same list and charges: one
        // evaluation gives both results
        if (smem)
            k_cs_coulomb<true><<<1, 1024, shb, s>>>(dd, dq, n, cf);
        else
            k_cs_coulomb<false><<<1, 1024, 0, s>>>(dd, dq, n, cf);
        float* frame = poslog ? dlog + pending * (int64_t)n3 : nullptr;
        k_cs_step<<<ga, 256, 0, s>>>(dx, dv, dF, dFn, dm, ljthr, ljall, cf, n, dt, dt2, lo, hi,
                                      frame);
        c->launches += 3;
        if (n > 1) {
            k_cs_pairs<<<n - 1, 256, 0, s>>>(dx, n, dd);  // update_pairslist!
            c->launches++;
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
