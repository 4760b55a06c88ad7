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
// LJ: each atom's additions are independent of other atoms' -- the pairs are
// sorted by i (stable, so each atom keeps its list order) and one thread per
// atom adds its run.  Coulomb: every update reads the result of earlier ones
// through force[i] and force[j]; the recurrence runs on one thread in list
// order (no parallel form reproduces its roundings).
#include <algorithm>
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

}  // namespace

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
