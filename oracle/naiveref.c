/*
 * naiveref.c -- CPU oracle (test infrastructure only, never shipped) for the
 * NaiveDynamics.jl hot path: LBVH neighbour search (src/Neighbors/BVHTraverse.jl),
 * brute-force pairs (src/Neighbors/AllToAll.jl) and an FP64 physics oracle for
 * the intended LJ + Coulomb forces and velocity-Verlet integrator
 * (src/Forces.jl, src/Simulator.jl).
 *
 * Build flags must keep IEEE single precision semantics exactly as Julia does:
 * no fast-math, no FMA contraction (-ffp-contract=off).
 */
#include "naiveref.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int ref_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ helpers */

/* Julia's min/max on IEEE floats (Base.min / Base.max): the sign of x - y picks
 * the argument, so -0.0 orders below +0.0 and the argument order is kept. */
static inline float jl_min(float x, float y) {
    float d = x - y;
    if (isnan(x) || isnan(y)) return d;
    return signbit(d) ? x : y;
}
static inline float jl_max(float x, float y) {
    float d = x - y;
    if (isnan(x) || isnan(y)) return d;
    return signbit(d) ? y : x;
}

float ref_dist2(const float* a, const float* b) {
    /* sum((a - b).^2) for SVector{3,Float32}: StaticArrays unrolls the sum
     * left to right, Julia emits plain fmul/fadd (no contraction). */
    float dx = a[0] - b[0];
    float dy = a[1] - b[1];
    float dz = a[2] - b[2];
    float sx = dx * dx;
    float sy = dy * dy;
    float sz = dz * dz;
    float s = sx + sy;
    return s + sz;
}

/* ---------------------------------------------------------------- spec / codes */

int ref_spec(int64_t atom_count, int64_t atomsperleaf, int32_t* leaves, int32_t* branches) {
    /* SpheresBVHSpecs (BVHTraverse.jl:71-94): apl must divide N, >= 2 leaves. */
    if (atomsperleaf <= 0 || atom_count <= 0 || atom_count > 2147483647LL) return REF_ERR_SPEC;
    if (atom_count % atomsperleaf != 0) return REF_ERR_SPEC;
    int64_t nl = atom_count / atomsperleaf;
    if (nl < 2) return REF_ERR_SPEC;
    if (leaves) *leaves = (int32_t)nl;
    if (branches) *branches = (int32_t)(nl - 1);
    return REF_OK;
}

int ref_morton_reference(const float* xyz, int64_t n, int32_t* codes) {
    /* BVHTraverse.jl:241-283: q = round(Int32, p / binwidth, RoundDown);
     * code |= (q & magic) & (q | ~magic) == q & magic, per axis. */
    const float binwidth = (float)(1.0 / 1023.0); /* Float32(1/1023), :184 */
    const int32_t magic[3] = {153391689, 306783378, 613566756};
    for (int64_t a = 0; a < n; ++a) {
        int32_t code = 0;
        for (int d = 0; d < 3; ++d) {
            float p = xyz[3 * a + d];
            if (!isfinite(p)) return REF_ERR_NONFINITE;
            float q = floorf(p / binwidth);
            /* trunc(Int32, ::Float32) accepts -2^31 <= x < 2^31 (Base float.jl). */
            if (!(q >= -2147483648.0f && q < 2147483648.0f)) return REF_ERR_RANGE;
            int32_t qi = (int32_t)q;
            int32_t yin = qi & magic[d];
            int32_t yang = qi | ~magic[d];
            code |= (yin & yang);
        }
        codes[a] = code;
    }
    return REF_OK;
}

/* 3-D Hilbert index of a cell of a 1024^3 grid: J. Skilling's transpose
 * method ("Programming the Hilbert curve", AIP Conf. Proc. 707, 2004), x
 * first in the interleave.  Consecutive indices are face-adjacent cells. */
static uint32_t hilbert3_10(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t X[3] = {x & 1023u, y & 1023u, z & 1023u};
    for (uint32_t Q = 1u << 9; Q > 1u; Q >>= 1) {
        uint32_t P = Q - 1u;
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                uint32_t t = (X[0] ^ X[i]) & P;
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
    for (int i = 0; i < 3; ++i) X[i] ^= t;
    uint32_t h = 0;
    for (int q = 9; q >= 0; --q)
        for (int i = 0; i < 3; ++i) h = (h << 1) | ((X[i] >> q) & 1u);
    return h;
}

uint32_t ref_hilbert3(uint32_t x, uint32_t y, uint32_t z) { return hilbert3_10(x, y, z); }

int ref_morton_spatial(const float* xyz, int64_t n, int32_t* codes) {
    /* Spatial code: 3-D Hilbert index over the Float32 bounding box, 1024 bins
     * per axis: s = 1024 / (hi - lo); q = clamp(floor((p - lo) * s), 0, 1023). */
    float lo[3], hi[3], s[3];
    for (int d = 0; d < 3; ++d) { lo[d] = INFINITY; hi[d] = -INFINITY; }
    for (int64_t a = 0; a < n; ++a)
        for (int d = 0; d < 3; ++d) {
            float p = xyz[3 * a + d];
            if (!isfinite(p)) return REF_ERR_NONFINITE;
            lo[d] = fminf(lo[d], p);
            hi[d] = fmaxf(hi[d], p);
        }
    for (int d = 0; d < 3; ++d) {
        float ext = hi[d] - lo[d];
        s[d] = (ext > 0.0f) ? 1024.0f / ext : 0.0f;
    }
    for (int64_t a = 0; a < n; ++a) {
        uint32_t q[3];
        for (int d = 0; d < 3; ++d) {
            float t = (xyz[3 * a + d] - lo[d]) * s[d];
            t = floorf(t);
            int32_t qi = (t < 0.0f) ? 0 : (t > 1023.0f ? 1023 : (int32_t)t);
            q[d] = (uint32_t)qi;
        }
        codes[a] = (int32_t)hilbert3_10(q[0], q[1], q[2]);
    }
    return REF_OK;
}

typedef struct { int32_t code; int32_t idx; } ci_pair;

static int ci_cmp(const void* pa, const void* pb) {
    const ci_pair* a = (const ci_pair*)pa;
    const ci_pair* b = (const ci_pair*)pb;
    if (a->code != b->code) return (a->code < b->code) ? -1 : 1;
    return (a->idx < b->idx) ? -1 : (a->idx > b->idx);
}

int ref_sortperm(const int32_t* codes, int64_t n, int32_t* perm) {
    /* sortperm is stable: equal codes keep ascending original index. */
    ci_pair* tmp = (ci_pair*)malloc(sizeof(ci_pair) * (size_t)(n > 0 ? n : 1));
    if (!tmp) return REF_ERR_NOMEM;
    for (int64_t i = 0; i < n; ++i) { tmp[i].code = codes[i]; tmp[i].idx = (int32_t)i; }
    qsort(tmp, (size_t)n, sizeof(ci_pair), ci_cmp);
    for (int64_t i = 0; i < n; ++i) perm[i] = tmp[i].idx;
    free(tmp);
    return REF_OK;
}

/* ----------------------------------------------------------------- tree build */

int32_t ref_delta(int32_t i, const int32_t* code_sorted, int32_t nL, int32_t apl) {
    /* exptdelta (BVHTraverse.jl:677-696), Int32 wrap-around arithmetic. */
    if (i >= nL || i < 1) return INT32_MAX;
    int32_t a = code_sorted[(int64_t)(i - 1) * apl]; /* atom 1 + (i-1)*apl */
    int32_t b = code_sorted[(int64_t)i * apl];       /* atom 1 + i*apl     */
    uint32_t x = (uint32_t)(a ^ b);
    uint32_t add = (x == 0u) ? (0x80000000u + (uint32_t)(i ^ (i + 1))) : 0u;
    return (int32_t)(x + add - 1u);
}

#define KEY(k) keys[(k) - 1]

static void bvh_interior(ref_key* keys, int32_t* store, int32_t i, int32_t nL,
                         const int32_t* code, int32_t apl) {
    /* bvh_interior! (BVHTraverse.jl:704-846); store is 1-based (store[s-1]). */
    int32_t rangel = i, ranger = i;
    int32_t dell = ref_delta(rangel - 1, code, nL, apl);
    int32_t delr = ref_delta(ranger, code, nL, apl);
    float bmin[3], bmax[3];
    for (int d = 0; d < 3; ++d) { bmin[d] = KEY(i).min[d]; bmax[d] = KEY(i).max[d]; }

    if (i == nL) {
        KEY(i).skip = 0;
    } else {
        int32_t ir = i + 1;
        KEY(i).skip = (delr < ref_delta(ir, code, nL, apl)) ? ir : nL + ir;
    }

    for (;;) {
        int32_t leftChild;
        if (delr < dell) {
            leftChild = i;
            int32_t split = ranger;
            int32_t old = store[split - 1];
            if (old == 0) { store[split - 1] = rangel; }
            ranger = old;
            if (ranger == 0) break;
            delr = ref_delta(ranger, code, nL, apl);
            int32_t rightChild = split + 1;
            if (rightChild != ranger) rightChild = nL + rightChild;
            for (int d = 0; d < 3; ++d) {
                bmax[d] = jl_max(KEY(rightChild).max[d], bmax[d]);
                bmin[d] = jl_min(KEY(rightChild).min[d], bmin[d]);
            }
        } else {
            int32_t split = rangel - 1;
            int32_t old = store[split - 1];
            if (old == 0) { store[split - 1] = ranger; }
            rangel = old;
            if (rangel == 0) break;
            dell = ref_delta(rangel - 1, code, nL, apl);
            leftChild = split;
            if (leftChild != rangel) leftChild = nL + leftChild;
            for (int d = 0; d < 3; ++d) {
                bmax[d] = jl_max(KEY(leftChild).max[d], bmax[d]);
                bmin[d] = jl_min(KEY(leftChild).min[d], bmin[d]);
            }
        }
        int32_t q = (delr < dell) ? ranger : rangel;
        int32_t parent = nL + q;
        int32_t skip;
        if (ranger == nL) {
            skip = 0;
        } else {
            int32_t r = ranger + 1;
            skip = (delr < ref_delta(r, code, nL, apl)) ? r : nL + r;
        }
        for (int d = 0; d < 3; ++d) { KEY(parent).min[d] = bmin[d]; KEY(parent).max[d] = bmax[d]; }
        KEY(parent).left = leftChild;
        KEY(parent).skip = skip;
        i = parent;
        if (i == nL + 1) return;
    }
}

static int tree_in_order(const float* xyz, int32_t n, float r, int32_t apl, int32_t boxes,
                         int32_t overwrite_root, ref_key* keys, int64_t nkeys,
                         const int32_t* idx_sorted, const int32_t* code_sorted, float* pos_sorted,
                         int32_t* store);

int ref_tree(const float* xyz, int32_t n, float r, int32_t apl, int32_t order, int32_t boxes,
             int32_t overwrite_root, ref_key* keys, int64_t nkeys, int32_t* idx_sorted,
             int32_t* code_sorted, float* pos_sorted, int32_t* perm) {
    int32_t nL = 0, nB = 0;
    int st = ref_spec(n, apl, &nL, &nB);
    if (st != REF_OK) return st;
    int64_t need = 2LL * nL - 1;
    if (boxes == REF_BOX_LEAF && (int64_t)n - 1 < need) return REF_ERR_SPEC; /* BoundsError in the reference */
    if (nkeys < need) return REF_ERR_ARG;

    int32_t* codes = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* store = (int32_t*)calloc((size_t)nB, sizeof(int32_t));
    if (!codes || !store) { free(codes); free(store); return REF_ERR_NOMEM; }
    st = (order == REF_ORDER_SPATIAL) ? ref_morton_spatial(xyz, n, codes)
                                      : ref_morton_reference(xyz, n, codes);
    if (st == REF_OK) st = ref_sortperm(codes, n, perm);
    if (st != REF_OK) { free(codes); free(store); return st; }

    for (int32_t k = 0; k < n; ++k) {
        int32_t o = perm[k];
        idx_sorted[k] = o + 1;
        code_sorted[k] = codes[o];
    }
    free(codes);
    st = tree_in_order(xyz, n, r, apl, boxes, overwrite_root, keys, nkeys, idx_sorted,
                       code_sorted, pos_sorted, store);
    free(store);
    return st;
}

/* The tree of positions xyz in a given sorted order (1-based original index
 * per sorted slot) with given sorted codes: leaf boxes, then the Apetrei
 * build, which depends on the sorted codes only.  With the order and codes of
 * an earlier build this is that build's topology with the boxes of the new
 * positions (the refit TreeData!, BVHTraverse.jl:601-655, intends). */
static int tree_in_order(const float* xyz, int32_t n, float r, int32_t apl, int32_t boxes,
                         int32_t overwrite_root, ref_key* keys, int64_t nkeys,
                         const int32_t* idx_sorted, const int32_t* code_sorted, float* pos_sorted,
                         int32_t* store) {
    int32_t nL = n / apl;
    for (int32_t k = 0; k < n; ++k) {
        int32_t o = idx_sorted[k] - 1;
        for (int d = 0; d < 3; ++d) pos_sorted[3 * k + d] = xyz[3 * o + d];
    }
    memset(keys, 0, sizeof(ref_key) * (size_t)nkeys);
    /* leafcluster_primitives (:376-410) uses r/2, cluster_primitives (:341-375) r. */
    float h = (boxes == REF_BOX_LEAF) ? r / 2.0f : r;
    for (int32_t leaf = 1; leaf <= nL; ++leaf) {
        int32_t bird = (leaf - 1) * apl; /* 0-based first atom */
        ref_key* k = &KEY(leaf);
        for (int d = 0; d < 3; ++d) {
            k->min[d] = pos_sorted[3 * bird + d] - h;
            k->max[d] = pos_sorted[3 * bird + d] + h;
        }
        for (int32_t i = 0; i < apl; ++i) {
            int32_t a = bird + i;
            for (int d = 0; d < 3; ++d) {
                k->min[d] = jl_min(k->min[d], pos_sorted[3 * a + d] - h);
                k->max[d] = jl_max(k->max[d], pos_sorted[3 * a + d] + h);
            }
        }
        k->left = 0;
        k->skip = 0;
    }
    /* bounding_volume_hierarchy! (:849-860): one task per leaf; running them in
     * leaf order is one valid interleaving of the CAS protocol. */
    for (int32_t i = 1; i <= nL; ++i) bvh_interior(keys, store, i, nL, code_sorted, apl);
    if (overwrite_root) {
        for (int d = 0; d < 3; ++d) { KEY(nL + 1).min[d] = 0.0f; KEY(nL + 1).max[d] = 1.0f; }
    }
    return REF_OK;
}

int ref_tree_kept(const float* xyz, int32_t n, float r, int32_t apl, int32_t overwrite_root,
                  ref_key* keys, int64_t nkeys, const int32_t* idx_sorted,
                  const int32_t* code_sorted, float* pos_sorted) {
    int32_t nL = 0, nB = 0;
    int st = ref_spec(n, apl, &nL, &nB);
    if (st != REF_OK) return st;
    if ((int64_t)n - 1 < 2LL * nL - 1 || nkeys < 2LL * nL - 1) return REF_ERR_SPEC;
    int32_t* store = (int32_t*)calloc((size_t)nB, sizeof(int32_t));
    if (!store) return REF_ERR_NOMEM;
    st = tree_in_order(xyz, n, r, apl, REF_BOX_LEAF, overwrite_root, keys, nkeys, idx_sorted,
                       code_sorted, pos_sorted, store);
    free(store);
    return st;
}

/* ------------------------------------------------------------------ traversal */

static inline int aabb_overlap(const ref_key* a, const ref_key* b) {
    /* aabb_overlap_test (BVHTraverse.jl:1094-1098): strict, all three axes. */
    int ok = 1;
    for (int d = 0; d < 3; ++d) ok &= (a->min[d] < b->max[d]) & (a->max[d] > b->min[d]);
    return ok;
}

#define EMIT(I, J, D)                                          \
    do {                                                       \
        if (count < cap) { pi[count] = (I); pj[count] = (J); pd[count] = (D); } \
        ++count;                                               \
    } while (0)

/* criterion 0: d^2 < r^2 (leafneighbor_traverse, BVHTraverse.jl:1048);
 * criterion 1: sqrt(d^2) < r (simdonecluster_proximitytest! /
 * simdtwocluster_proximitytest!, ext/NaiveSIMD.jl:529,589), with the same
 * tree, traversal and emission order (simdneighbor_traverse, :610-704, on one
 * thread). */
static inline int pair_hit(float d2, float r, float r2, int32_t criterion) {
    return criterion == 0 ? (d2 < r2) : (sqrtf(d2) < r);
}

int64_t ref_leaf_traverse_crit(const ref_key* keys, const int32_t* idx, const float* pos,
                               int32_t nL, int32_t apl, float r, int32_t criterion, int32_t* pi,
                               int32_t* pj, float* pd, int64_t cap);

int64_t ref_leaf_traverse(const ref_key* keys, const int32_t* idx, const float* pos, int32_t nL,
                          int32_t apl, float r, int32_t* pi, int32_t* pj, float* pd, int64_t cap) {
    return ref_leaf_traverse_crit(keys, idx, pos, nL, apl, r, 0, pi, pj, pd, cap);
}

int64_t ref_leaf_traverse_crit(const ref_key* keys, const int32_t* idx, const float* pos,
                               int32_t nL, int32_t apl, float r, int32_t criterion, int32_t* pi,
                               int32_t* pj, float* pd, int64_t cap) {
    const float r2 = r * r;
    int64_t count = 0;
    for (int32_t q = 1; q <= nL; ++q) {
        const ref_key* ql = &KEY(q);
        int32_t A = (q - 1) * apl;
        /* onecluster_proximitytest! (:1021-1040) */
        for (int32_t i = 0; i < apl - 1; ++i)
            for (int32_t j = i + 1; j < apl; ++j) {
                float d2 = ref_dist2(&pos[3 * (A + i)], &pos[3 * (A + j)]);
                if (pair_hit(d2, r, r2, criterion)) EMIT(idx[A + i], idx[A + j], sqrtf(d2));
            }
        int32_t t = ql->skip;
        while (t != 0) {
            const ref_key* node = &KEY(t);
            if (aabb_overlap(ql, node)) {
                if (node->left == 0) {
                    int32_t B = (t - 1) * apl;
                    /* twocluster_proximitytest! (:1042-1055) */
                    for (int32_t i = 0; i < apl; ++i)
                        for (int32_t j = 0; j < apl; ++j) {
                            float d2 = ref_dist2(&pos[3 * (A + i)], &pos[3 * (B + j)]);
                            if (pair_hit(d2, r, r2, criterion)) EMIT(idx[A + i], idx[B + j], sqrtf(d2));
                        }
                    t = node->skip;
                } else {
                    t = node->left;
                }
            } else {
                t = node->skip;
            }
        }
    }
    return count;
}

static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline void hash_one(int32_t i, int32_t j, float d, uint64_t* h0, uint64_t* h1) {
    uint32_t a = (uint32_t)(i < j ? i : j);
    uint32_t b = (uint32_t)(i < j ? j : i);
    uint32_t db;
    memcpy(&db, &d, 4);
    uint64_t k = ((uint64_t)a << 32) | (uint64_t)b;
    uint64_t x = mix64(k ^ ((uint64_t)db * 0xD6E8FEB86659FD93ull));
    uint64_t y = mix64(x ^ ((uint64_t)db << 21) ^ 0x5851F42D4C957F2Dull);
    *h0 += x;
    *h1 += y;
}

void ref_pair_hash(const int32_t* pi, const int32_t* pj, const float* pd, int64_t np,
                   uint64_t hash_out[2]) {
    uint64_t h0 = 0, h1 = 0;
    for (int64_t k = 0; k < np; ++k) hash_one(pi[k], pj[k], pd[k], &h0, &h1);
    hash_out[0] = h0;
    hash_out[1] = h1;
}

int64_t ref_leaf_traverse_hash(const ref_key* keys, const int32_t* idx, const float* pos,
                               int32_t nL, int32_t apl, float r, uint64_t hash_out[2]) {
    const float r2 = r * r;
    int64_t total = 0;
    uint64_t H0 = 0, H1 = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total, H0, H1)
    for (int32_t q = 1; q <= nL; ++q) {
        const ref_key* ql = &KEY(q);
        int32_t A = (q - 1) * apl;
        uint64_t h0 = 0, h1 = 0;
        int64_t c = 0;
        for (int32_t i = 0; i < apl - 1; ++i)
            for (int32_t j = i + 1; j < apl; ++j) {
                float d2 = ref_dist2(&pos[3 * (A + i)], &pos[3 * (A + j)]);
                if (d2 < r2) { hash_one(idx[A + i], idx[A + j], sqrtf(d2), &h0, &h1); ++c; }
            }
        int32_t t = ql->skip;
        while (t != 0) {
            const ref_key* node = &KEY(t);
            if (aabb_overlap(ql, node)) {
                if (node->left == 0) {
                    int32_t B = (t - 1) * apl;
                    for (int32_t i = 0; i < apl; ++i)
                        for (int32_t j = 0; j < apl; ++j) {
                            float d2 = ref_dist2(&pos[3 * (A + i)], &pos[3 * (B + j)]);
                            if (d2 < r2) { hash_one(idx[A + i], idx[B + j], sqrtf(d2), &h0, &h1); ++c; }
                        }
                    t = node->skip;
                } else {
                    t = node->left;
                }
            } else {
                t = node->skip;
            }
        }
        total += c;
        H0 += h0;
        H1 += h1;
    }
    hash_out[0] = H0;
    hash_out[1] = H1;
    return total;
}

int64_t ref_atom_traverse(const ref_key* keys, const int32_t* idx, const float* pos, int32_t n,
                          int32_t apl, float r, int32_t* pi, int32_t* pj, float* pd, int64_t cap) {
    /* neighbor_traverse (:1125-1183): queries 1..N-1 start at their own leaf
     * ceil(q/apl); point-in-box test overlap_test (:1089-1092); a leaf emits
     * subjects s with q < s (proximity_test!, :1057-1086). */
    const float r2 = r * r;
    int64_t count = 0;
    for (int32_t qi = 1; qi <= n - 1; ++qi) {
        const float* p = &pos[3 * (qi - 1)];
        int32_t t = (qi + apl - 1) / apl;
        while (t != 0) {
            const ref_key* node = &KEY(t);
            int in = 1;
            for (int d = 0; d < 3; ++d) in &= (node->min[d] < p[d]) & (p[d] < node->max[d]);
            if (in) {
                if (node->left == 0) {
                    int32_t low = (t - 1) * apl + 1;
                    for (int32_t e = 1; e <= apl; ++e) {
                        int32_t s = low + e - 1;
                        if (qi < e + low && idx[qi - 1] != idx[s - 1]) {
                            float d2 = ref_dist2(p, &pos[3 * (s - 1)]);
                            if (d2 < r2) EMIT(idx[qi - 1], idx[s - 1], sqrtf(d2));
                        }
                    }
                    t = node->skip;
                } else {
                    t = node->left;
                }
            } else {
                t = node->skip;
            }
        }
    }
    return count;
}

int64_t ref_brute_pairs(const float* xyz, int32_t n, float r, int32_t criterion, int32_t* pi,
                        int32_t* pj, float* pd, int64_t cap) {
    const float r2 = r * r;
    int64_t count = 0;
    for (int32_t i = 0; i < n - 1; ++i)
        for (int32_t j = i + 1; j < n; ++j) {
            float d2 = ref_dist2(&xyz[3 * i], &xyz[3 * j]);
            float d = sqrtf(d2);
            int hit = (criterion == 0) ? (d2 < r2) : (d < r);
            if (hit) EMIT(i + 1, j + 1, d);
        }
    return count;
}

/* ------------------------------------------------- bug-compatible force calls */

/* Julia's Base.Math.pow_body(x::Float64, n::Integer), n >= 4: power by
 * squaring carrying the low part of every product (two_mul), muladd fused. */
static double jl_pow_int(double x, int n) {
    double y = 1.0, xnlo = 0.0, ynlo = 0.0;
    while (n > 1) {
        if (n & 1) {
            double err = fma(y, xnlo, x * ynlo);
            double yy = x * y;
            ynlo = fma(x, y, -yy) + err;
            y = yy;
        }
        double err = x * 2.0 * xnlo;
        double xx = x * x;
        xnlo = fma(x, x, -xx) + err;
        x = xx;
        n >>= 1;
    }
    double err = fma(y, xnlo, x * ynlo);
    return (isfinite(x) && isfinite(err)) ? fma(x, y, err) : x * y;
}

/* force_lennardjones! (Forces.jl:6-45) over the list in order. */
void ref_compat_force_lj(int32_t n, const int32_t* pi, const int32_t* pj, const float* pd,
                         int64_t np, float* force) {
    const float eps = -1e10f;
    const double sigma = 0.0001;
    memset(force, 0, sizeof(float) * 3 * (size_t)n);
    for (int64_t p = 0; p < np; ++p) {
        const int32_t i = pi[p] - 1;
        const float d = pd[p];
        const float a = (24.0f * eps) / d;
        const double b = jl_pow_int(2.0 * sigma / (double)d, 12);
        const double c = jl_pow_int(sigma / (double)d, 6);
        const double x = (double)a * (b - c);
        for (int k = 0; k < 3; ++k) force[3 * i + k] = (float)((double)force[3 * i + k] + x);
    }
}

/* force_coulomb! (Forces.jl:46-66) over the list in order. */
void ref_compat_force_coulomb(int32_t n, const int32_t* pi, const int32_t* pj, const float* pd,
                              int64_t np, const float* q, float* force) {
    memset(force, 0, sizeof(float) * 3 * (size_t)n);
    for (int64_t p = 0; p < np; ++p) {
        const int32_t i = pi[p] - 1, j = pj[p] - 1;
        const float d = pd[p];
        const float add = (1.0f * q[i]) * q[j] / (d * d);
        for (int k = 0; k < 3; ++k) force[3 * i + k] += add;
        for (int k = 0; k < 3; ++k) force[3 * j + k] -= force[3 * i + k];
    }
}

/* update_pairslist! (AllToAll.jl:7-62): d = sqrt(sum((a[i] .- a[j]) .^ 2)). */
static void compat_update_pairs(const float* x, const int32_t* pi, const int32_t* pj, float* pd,
                                int64_t np) {
    for (int64_t p = 0; p < np; ++p) {
        const float* a = &x[3 * (pi[p] - 1)];
        const float* b = &x[3 * (pj[p] - 1)];
        const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
        pd[p] = sqrtf(dx * dx + dy * dy + dz * dz);
    }
}

/* rescale_velocity! (Simulator.jl:119-144); 1 on DomainError. */
static int compat_rescale(float* v, float Tf, float gamma, const float* mass, int32_t n,
                          int64_t objectcount) {
    float Ti = 0.0f;
    const float kb = 1.0f;
    const float objects = (float)objectcount;
    for (int32_t k = 0; k < n; ++k) {
        const float* w = &v[3 * k];
        /* (v1^2 + v2^2 + v3^2) ^ 0.5 promoted to Float64, stored as Float32 */
        const float s = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
        const float vv = (float)sqrt((double)s);
        Ti += (2.0f / (3.0f * objects * kb)) * vv * mass[k] / 2.0f;
    }
    const float r = 1.0f + gamma * (Tf / Ti - 1.0f);
    if (r < 0.0f) return 1;
    const double beta = sqrt((double)r);
    for (int64_t e = 0; e < 3 * (int64_t)n; ++e) v[e] = (float)((double)v[e] * beta);
    return 0;
}

int ref_compat_simulate(const ref_compat_sim* spec, int32_t n, float* x, float* v, float* force,
                        const float* mass, const float* q, float* poslog) {
    if (n < 1) return 0;
    const size_t n3 = 3 * (size_t)n;
    const int64_t np = (int64_t)n * (n - 1) / 2;
    int32_t* pi = (int32_t*)malloc(sizeof(int32_t) * (size_t)(np + 1));
    int32_t* pj = (int32_t*)malloc(sizeof(int32_t) * (size_t)(np + 1));
    float* pd = (float*)malloc(sizeof(float) * (size_t)(np + 1));
    int32_t* ti = (int32_t*)malloc(sizeof(int32_t) * (size_t)(np + 1));
    int32_t* tj = (int32_t*)malloc(sizeof(int32_t) * (size_t)(np + 1));
    float* td = (float*)malloc(sizeof(float) * (size_t)(np + 1));
    float* fnext = (float*)malloc(sizeof(float) * n3);
    float* flj = (float*)malloc(sizeof(float) * n3);
    float* fc = (float*)malloc(sizeof(float) * n3);
    float* at = (float*)malloc(sizeof(float) * n3);
    float* atdt = (float*)malloc(sizeof(float) * n3);
    int status = 0;
    const float dt = (float)spec->stepwidth;
    const float dt2 = (float)(int64_t)((uint64_t)spec->stepwidth * (uint64_t)spec->stepwidth);
    memcpy(fnext, force, sizeof(float) * n3); /* force_nextstep = deepcopy(sys.force) */
    /* pairslist = unique_pairs(sys.position) (AllToAll.jl:65-80) */
    int64_t p = 0;
    for (int32_t i = 1; i <= n - 1; ++i)
        for (int32_t j = i + 1; j <= n; ++j) {
            pi[p] = i;
            pj[p] = j;
            ++p;
        }
    compat_update_pairs(x, pi, pj, pd, np);
    for (int64_t step = 1; step <= spec->duration; ++step) {
        /* LJ_pairs = threshold_pairs(pairslist, 0.01) */
        int64_t nt = 0;
        for (int64_t k = 0; k < np; ++k)
            if (pd[k] < 0.01f) {
                ti[nt] = pi[k];
                tj[nt] = pj[k];
                td[nt] = pd[k];
                ++nt;
            }
        ref_compat_force_lj(n, ti, tj, td, nt, flj);
        ref_compat_force_coulomb(n, pi, pj, pd, np, q, fc);
        for (size_t e = 0; e < n3; ++e) force[e] = flj[e] + fc[e]; /* sum_forces! */
        for (size_t e = 0; e < n3; ++e) at[e] = force[e] / mass[e / 3];
        for (size_t e = 0; e < n3; ++e) x[e] += v[e] * dt + ((at[e] * dt2) / 2.0f);
        for (size_t e = 0; e < n3; ++e) atdt[e] = fnext[e] / mass[e / 3];
        memcpy(fnext, force, sizeof(float) * n3);
        ref_compat_force_lj(n, pi, pj, pd, np, flj);
        ref_compat_force_coulomb(n, pi, pj, pd, np, q, fc);
        for (size_t e = 0; e < n3; ++e) fnext[e] = flj[e] + fc[e];
        for (size_t e = 0; e < n3; ++e) v[e] += ((at[e] + atdt[e]) * dt) / 2.0f;
        /* boundary_reflect! (Simulator.jl:81-111) */
        for (int32_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                float* xk = &x[3 * i + k];
                float* vk = &v[3 * i + k];
                if (spec->min_dim[k] > *xk) {
                    *vk *= -1.0f;
                    *xk = spec->min_dim[k];
                }
                if (spec->max_dim[k] < *xk) {
                    *vk *= -1.0f;
                    *xk = spec->max_dim[k];
                }
            }
        memcpy(force, fnext, sizeof(float) * n3);
        compat_update_pairs(x, pi, pj, pd, np);
        if (step % 10 == 0 &&
            compat_rescale(v, spec->temperature, spec->velocity_dampening, mass, n,
                           spec->objectnumber)) {
            status = 1;
            break;
        }
        if (poslog) memcpy(poslog + step * (int64_t)n3, x, sizeof(float) * n3);
    }
    if (poslog && status == 0) memcpy(poslog, x, sizeof(float) * n3);
    free(pi), free(pj), free(pd), free(ti), free(tj), free(td);
    free(fnext), free(flj), free(fc), free(at), free(atdt);
    return status;
}

/* collect_objects (MDInput.jl:305-369).  Draw k of stream c is
 * mix64(seed ^ mix64(c << 56 ^ k)); Uniform(a, b) = a + (b - a) u, u of 53
 * bits, stored as Float32; rand(Float32) of 24 bits. */
static uint64_t cobj_bits(uint64_t seed, uint64_t stream, uint64_t k) {
    return mix64(seed ^ mix64((stream << 56) ^ k));
}
static float cobj_uniform(uint64_t seed, uint64_t stream, uint64_t k, float a, float b) {
    const double u = (double)(cobj_bits(seed, stream, k) >> 11) * 0x1.0p-53;
    return (float)((double)a + (double)(b - a) * u);
}

int64_t ref_collect_objects(const ref_collector* cl, uint64_t seed, float* x, float* v, float* m,
                            float* q) {
    const int64_t n = cl->objectnumber;
    float* vd = (float*)malloc(sizeof(float) * 3 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        m[i] = cobj_uniform(seed, 0, (uint64_t)i, cl->minmass, cl->maxmass);
        q[i] = cobj_uniform(seed, 1, (uint64_t)i, cl->mincharge, cl->maxcharge);
        for (int d = 0; d < 3; ++d) {
            x[3 * i + d] = cobj_uniform(seed, 2 + d, (uint64_t)i, cl->min_dim[d], cl->max_dim[d]);
            vd[d * n + i] = (float)(cobj_bits(seed, 5 + d, (uint64_t)i) >> 40) * 0x1.0p-24f;
        }
    }
    /* sum(veldist): 256-element chunks as a binary tree, chunk sums in order */
    float sum[3] = {0.0f, 0.0f, 0.0f};
    for (int d = 0; d < 3; ++d)
        for (int64_t c0 = 0; c0 < n; c0 += 256) {
            float t[256];
            for (int k = 0; k < 256; ++k) t[k] = c0 + k < n ? vd[d * n + c0 + k] : 0.0f;
            for (int w = 128; w > 0; w >>= 1)
                for (int k = 0; k < w; ++k) t[k] = t[k] + t[k + w];
            sum[d] = sum[d] + t[0];
        }
    const float N = (float)n;
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            const float a = cl->randomvelocity
                                ? cl->temperature * (vd[d * n + i] / sum[d]) * 3.0f * N
                                : cl->temperature / N * 3.0f * N;
            v[3 * i + d] = a * 1.0f / m[i];
        }
    free(vd);
    /* unique_pairs_prune (MDInput.jl:228-259) as written */
    int64_t tooClose = 0;
    for (int64_t i = 1; i <= n - 1; ++i)
        for (int64_t j = i + 1; j <= n - 1; ++j) {
            float* a = &x[3 * (i - 1)];
            const float* b = &x[3 * (j - 1)];
            const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
            const float d2 = sqrtf(dx * dx + dy * dy + dz * dz);
            if (d2 < cl->minimumdistance) {
                a[0] = a[1] = a[2] = INFINITY;
                tooClose += 1;
            }
        }
    return tooClose;
}

/* --------------------------------------------------------------- FP64 physics */

static inline void pair_force(const ref_md_params* p, const double* xi, const double* xj,
                              double qi, double qj, double fij[3], double* u, int* hit) {
    double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
    double r2 = dx * dx + dy * dy + dz * dz;
    *hit = 0;
    if (!(r2 < p->cutoff * p->cutoff)) return;
    *hit = 1;
    double inv_r2 = 1.0 / r2;
    double s2 = p->sigma * p->sigma * inv_r2;
    double s6 = s2 * s2 * s2;
    double fmag = 24.0 * p->epsilon * inv_r2 * (2.0 * s6 * s6 - s6);
    double e = 4.0 * p->epsilon * (s6 * s6 - s6);
    if (p->coulomb_k != 0.0) {
        double inv_r = 1.0 / sqrt(r2);
        double kqq = p->coulomb_k * qi * qj;
        fmag += kqq * inv_r * inv_r2;
        e += kqq * inv_r;
    }
    fij[0] = fmag * dx;
    fij[1] = fmag * dy;
    fij[2] = fmag * dz;
    *u = e;
}

int64_t ref_forces(const ref_md_params* p, int32_t n, const double* x, const double* q,
                   double* f, double* energy) {
    /* Cell list with cells >= cutoff over the bounding box of x. */
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) { lo[d] = INFINITY; hi[d] = -INFINITY; }
    for (int32_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            if (x[3 * i + d] < lo[d]) lo[d] = x[3 * i + d];
            if (x[3 * i + d] > hi[d]) hi[d] = x[3 * i + d];
        }
    int nc[3];
    double cs[3];
    int64_t ncell = 1;
    for (int d = 0; d < 3; ++d) {
        double ext = hi[d] - lo[d];
        int c = (int)floor(ext / p->cutoff);
        if (c < 1) c = 1;
        if (c > 1024) c = 1024;
        nc[d] = c;
        cs[d] = (ext > 0) ? ext / c : 1.0;
        ncell *= c;
    }
    int32_t* head = (int32_t*)malloc(sizeof(int32_t) * (size_t)ncell);
    int32_t* next = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* cell = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    if (!head || !next || !cell) { free(head); free(next); free(cell); return REF_ERR_NOMEM; }
    for (int64_t c = 0; c < ncell; ++c) head[c] = -1;
    for (int32_t i = n - 1; i >= 0; --i) {
        int ci[3];
        for (int d = 0; d < 3; ++d) {
            int c = (int)floor((x[3 * i + d] - lo[d]) / cs[d]);
            if (c < 0) c = 0;
            if (c >= nc[d]) c = nc[d] - 1;
            ci[d] = c;
        }
        int32_t id = (ci[2] * nc[1] + ci[1]) * nc[0] + ci[0];
        cell[i] = id;
        next[i] = head[id];
        head[id] = i;
    }
    memset(f, 0, sizeof(double) * 3 * (size_t)n);
    double U = 0.0;
    int64_t npairs = 0;
    for (int32_t i = 0; i < n; ++i) {
        int32_t id = cell[i];
        int cx = id % nc[0], cy = (id / nc[0]) % nc[1], cz = id / (nc[0] * nc[1]);
        for (int oz = -1; oz <= 1; ++oz)
            for (int oy = -1; oy <= 1; ++oy)
                for (int ox = -1; ox <= 1; ++ox) {
                    int X = cx + ox, Y = cy + oy, Z = cz + oz;
                    if (X < 0 || Y < 0 || Z < 0 || X >= nc[0] || Y >= nc[1] || Z >= nc[2]) continue;
                    for (int32_t j = head[(Z * nc[1] + Y) * nc[0] + X]; j >= 0; j = next[j]) {
                        if (j <= i) continue;
                        double fij[3], u;
                        int hit;
                        pair_force(p, &x[3 * i], &x[3 * j], q ? q[i] : 0.0, q ? q[j] : 0.0, fij, &u, &hit);
                        if (!hit) continue;
                        ++npairs;
                        U += u;
                        for (int d = 0; d < 3; ++d) { f[3 * i + d] += fij[d]; f[3 * j + d] -= fij[d]; }
                    }
                }
    }
    free(head); free(next); free(cell);
    if (energy) *energy = U;
    return npairs;
}

static void reflect(const ref_md_params* p, int32_t n, double* x, double* v) {
    /* boundary_reflect! (Simulator.jl:81-111): clamp to the wall, flip v. */
    for (int32_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            if (p->box_lo[d] > x[3 * i + d]) { v[3 * i + d] *= -1.0; x[3 * i + d] = p->box_lo[d]; }
            if (p->box_hi[d] < x[3 * i + d]) { v[3 * i + d] *= -1.0; x[3 * i + d] = p->box_hi[d]; }
        }
}

int ref_md_run(const ref_md_params* p, int32_t n, double* x, double* v, double* f,
               const double* q, const double* m, int64_t steps) {
    const double h = 0.5 * p->dt;
    for (int64_t s = 0; s < steps; ++s) {
        for (int32_t i = 0; i < n; ++i) {
            double im = m ? 1.0 / m[i] : 1.0;
            for (int d = 0; d < 3; ++d) {
                v[3 * i + d] += h * f[3 * i + d] * im;
                x[3 * i + d] += p->dt * v[3 * i + d];
            }
        }
        reflect(p, n, x, v);
        int64_t st = ref_forces(p, n, x, q, f, NULL);
        if (st < 0) return (int)st;
        for (int32_t i = 0; i < n; ++i) {
            double im = m ? 1.0 / m[i] : 1.0;
            for (int d = 0; d < 3; ++d) v[3 * i + d] += h * f[3 * i + d] * im;
        }
    }
    return REF_OK;
}

/* rescale_velocity! (Simulator.jl:119-144): Ti = sum_i (2/(3 N kb)) |v_i| m_i/2
 * with kb = 1 (the reference sums the speed, not its square), then
 * beta = (1 + gamma (Tf/Ti - 1))^0.5 and every velocity scaled by beta.
 * Ti <= 0 leaves the velocities unchanged. */
static void rescale_velocity(int32_t n, double* v, const double* m, double Tf, double gamma) {
    double Ti = 0.0;
    const double c = 2.0 / (3.0 * (double)n * 1.0);
    for (int32_t i = 0; i < n; ++i) {
        const double s = sqrt(v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] +
                              v[3 * i + 2] * v[3 * i + 2]);
        Ti += c * s * (m ? m[i] : 1.0) / 2.0;
    }
    if (!(Ti > 0.0)) return;
    const double beta = sqrt(1.0 + gamma * (Tf / Ti - 1.0));
    for (int64_t k = 0; k < 3 * (int64_t)n; ++k) v[k] *= beta;
}

int ref_md_run_observed(const ref_md_params* p, int32_t n, double* x, double* v, double* f,
                        const double* q, const double* m, int64_t steps, double thermo_T,
                        double thermo_gamma, int32_t thermo_every, int32_t log_every,
                        double* poslog) {
    const double h = 0.5 * p->dt;
    int64_t frame = 0;
    for (int64_t s = 1; s <= steps; ++s) {
        for (int32_t i = 0; i < n; ++i) {
            double im = m ? 1.0 / m[i] : 1.0;
            for (int d = 0; d < 3; ++d) {
                v[3 * i + d] += h * f[3 * i + d] * im;
                x[3 * i + d] += p->dt * v[3 * i + d];
            }
        }
        reflect(p, n, x, v);
        int64_t st = ref_forces(p, n, x, q, f, NULL);
        if (st < 0) return (int)st;
        for (int32_t i = 0; i < n; ++i) {
            double im = m ? 1.0 / m[i] : 1.0;
            for (int d = 0; d < 3; ++d) v[3 * i + d] += h * f[3 * i + d] * im;
        }
        /* simulate! (Simulator.jl:241-245): rescale every thermo_every steps,
         * then log the positions */
        if (thermo_every > 0 && s % thermo_every == 0)
            rescale_velocity(n, v, m, thermo_T, thermo_gamma);
        if (log_every > 0 && s % log_every == 0 && poslog) {
            memcpy(poslog + frame * 3 * (int64_t)n, x, sizeof(double) * 3 * (size_t)n);
            ++frame;
        }
    }
    return REF_OK;
}

/* CPU baseline: leaf BVH every `rebuild` steps + FP64 forces over the half list. */
typedef struct { int32_t* i; int32_t* j; int64_t n, cap; } pairbuf;

static int pb_push(pairbuf* b, int32_t i, int32_t j) {
    if (b->n == b->cap) {
        int64_t nc = b->cap ? 2 * b->cap : 1024;
        int32_t* ni = (int32_t*)realloc(b->i, sizeof(int32_t) * (size_t)nc);
        if (!ni) return -1;
        b->i = ni;
        int32_t* nj = (int32_t*)realloc(b->j, sizeof(int32_t) * (size_t)nc);
        if (!nj) return -1;
        b->j = nj;
        b->cap = nc;
    }
    b->i[b->n] = i;
    b->j[b->n] = j;
    ++b->n;
    return 0;
}

static int64_t build_half_list(const double* x, int32_t n, float rl, int32_t apl, int32_t order,
                               pairbuf* out) {
    int32_t nL, nB;
    if (ref_spec(n, apl, &nL, &nB) != REF_OK) return REF_ERR_SPEC;
    int64_t nkeys = 2LL * nL - 1;
    float* xf = (float*)malloc(sizeof(float) * 3 * (size_t)n);
    float* ps = (float*)malloc(sizeof(float) * 3 * (size_t)n);
    int32_t* idx = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* code = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* perm = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    ref_key* keys = (ref_key*)malloc(sizeof(ref_key) * (size_t)(nkeys > n ? nkeys : n));
    if (!xf || !ps || !idx || !code || !perm || !keys) return REF_ERR_NOMEM;
    for (int64_t k = 0; k < 3LL * n; ++k) xf[k] = (float)x[k];
    int st = ref_tree(xf, n, rl, apl, order, REF_BOX_LEAF, 1, keys, nkeys, idx, code, ps, perm);
    if (st != REF_OK) return st;
    const float r2 = rl * rl;
    int nt = ref_num_threads();
    pairbuf* bufs = (pairbuf*)calloc((size_t)nt, sizeof(pairbuf));
    /* leafneighbor_traverse (:1236-1323): strided query chunks per thread. */
#pragma omp parallel
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
        int nth = omp_get_num_threads();
#else
        int tid = 0, nth = 1;
#endif
        pairbuf* b = &bufs[tid];
        for (int32_t q = 1 + tid; q <= nL; q += nth) {
            const ref_key* ql = &KEY(q);
            int32_t A = (q - 1) * apl;
            for (int32_t i = 0; i < apl - 1; ++i)
                for (int32_t j = i + 1; j < apl; ++j)
                    if (ref_dist2(&ps[3 * (A + i)], &ps[3 * (A + j)]) < r2)
                        pb_push(b, idx[A + i] - 1, idx[A + j] - 1);
            int32_t t = ql->skip;
            while (t != 0) {
                const ref_key* node = &KEY(t);
                if (aabb_overlap(ql, node)) {
                    if (node->left == 0) {
                        int32_t B = (t - 1) * apl;
                        for (int32_t i = 0; i < apl; ++i)
                            for (int32_t j = 0; j < apl; ++j)
                                if (ref_dist2(&ps[3 * (A + i)], &ps[3 * (B + j)]) < r2)
                                    pb_push(b, idx[A + i] - 1, idx[B + j] - 1);
                        t = node->skip;
                    } else {
                        t = node->left;
                    }
                } else {
                    t = node->skip;
                }
            }
        }
    }
    out->n = 0;
    for (int t = 0; t < nt; ++t) {
        for (int64_t k = 0; k < bufs[t].n; ++k) pb_push(out, bufs[t].i[k], bufs[t].j[k]);
        free(bufs[t].i);
        free(bufs[t].j);
    }
    free(bufs); free(xf); free(ps); free(idx); free(code); free(perm); free(keys);
    return out->n;
}

static void forces_from_list(const ref_md_params* p, int32_t n, const double* x, const double* q,
                             const pairbuf* L, double* f, double* fth, int nt) {
#pragma omp parallel
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double* ft = fth + (size_t)tid * 3 * (size_t)n;
        memset(ft, 0, sizeof(double) * 3 * (size_t)n);
#pragma omp for schedule(static)
        for (int64_t k = 0; k < L->n; ++k) {
            int32_t i = L->i[k], j = L->j[k];
            double fij[3], u;
            int hit;
            pair_force(p, &x[3 * i], &x[3 * j], q ? q[i] : 0.0, q ? q[j] : 0.0, fij, &u, &hit);
            if (!hit) continue;
            for (int d = 0; d < 3; ++d) { ft[3 * i + d] += fij[d]; ft[3 * j + d] -= fij[d]; }
        }
#pragma omp for schedule(static)
        for (int64_t k = 0; k < 3LL * n; ++k) {
            double s = 0.0;
            for (int t = 0; t < nt; ++t) s += fth[(size_t)t * 3 * (size_t)n + (size_t)k];
            f[k] = s;
        }
    }
}

int64_t ref_md_run_bvh(const ref_md_params* p, int32_t n, double* x, double* v, double* f,
                       const double* q, const double* m, int64_t steps, int32_t rebuild,
                       double skin, int32_t apl, int32_t order) {
    int nt = ref_num_threads();
    double* fth = (double*)malloc(sizeof(double) * 3 * (size_t)n * (size_t)nt);
    if (!fth) return REF_ERR_NOMEM;
    pairbuf L = {0};
    const float rl = (float)(p->cutoff + skin);
    const double h = 0.5 * p->dt;
    int64_t st = build_half_list(x, n, rl, apl, order, &L);
    if (st < 0) { free(fth); return st; }
    forces_from_list(p, n, x, q, &L, f, fth, nt);
    for (int64_t s = 0; s < steps; ++s) {
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; ++i) {
            double im = m ? 1.0 / m[i] : 1.0;
            for (int d = 0; d < 3; ++d) {
                v[3 * i + d] += h * f[3 * i + d] * im;
                x[3 * i + d] += p->dt * v[3 * i + d];
            }
        }
        reflect(p, n, x, v);
        if (rebuild > 0 && (s + 1) % rebuild == 0) {
            st = build_half_list(x, n, rl, apl, order, &L);
            if (st < 0) break;
        }
        forces_from_list(p, n, x, q, &L, f, fth, nt);
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; ++i) {
            double im = m ? 1.0 / m[i] : 1.0;
            for (int d = 0; d < 3; ++d) v[3 * i + d] += h * f[3 * i + d] * im;
        }
    }
    int64_t np = L.n;
    free(L.i); free(L.j); free(fth);
    return st < 0 ? st : np;
}

/* ---------------------------------------------- steady-state CPU baseline */

/* The loop of ref_md_run_bvh as a session: creation copies the state, builds
 * the first list and evaluates the forces (the set-up a run pays once);
 * ref_md_bvh_steps then advances with the rebuild after every `rebuild`-th
 * step since creation, so a window of `rebuild` steps holds exactly one
 * leaf-BVH build and `rebuild` force evaluations. */
struct ref_md_bvh {
    ref_md_params p;
    int32_t n, rebuild, apl, order, nt;
    float rl;
    int64_t done;
    double *x, *v, *f, *q, *im, *fth;
    pairbuf L;
};

ref_md_bvh* ref_md_bvh_create(const ref_md_params* p, int32_t n, const double* x,
                              const double* v, const double* q, const double* m,
                              int32_t rebuild, double skin, int32_t apl, int32_t order) {
    ref_md_bvh* s = (ref_md_bvh*)calloc(1, sizeof(ref_md_bvh));
    if (!s) return NULL;
    s->p = *p;
    s->n = n;
    s->rebuild = rebuild;
    s->apl = apl;
    s->order = order;
    s->nt = ref_num_threads();
    s->rl = (float)(p->cutoff + skin);
    const size_t b = sizeof(double) * 3 * (size_t)n;
    s->x = (double*)malloc(b);
    s->v = (double*)malloc(b);
    s->f = (double*)malloc(b);
    s->q = q ? (double*)malloc(sizeof(double) * (size_t)n) : NULL;
    s->im = (double*)malloc(sizeof(double) * (size_t)n);
    s->fth = (double*)malloc(b * (size_t)s->nt);
    if (!s->x || !s->v || !s->f || (q && !s->q) || !s->im || !s->fth) {
        ref_md_bvh_destroy(s);
        return NULL;
    }
    memcpy(s->x, x, b);
    memcpy(s->v, v, b);
    if (q) memcpy(s->q, q, sizeof(double) * (size_t)n);
    for (int32_t i = 0; i < n; ++i) s->im[i] = m ? 1.0 / m[i] : 1.0;
    if (build_half_list(s->x, n, s->rl, apl, order, &s->L) < 0) {
        ref_md_bvh_destroy(s);
        return NULL;
    }
    forces_from_list(&s->p, n, s->x, s->q, &s->L, s->f, s->fth, s->nt);
    return s;
}

int64_t ref_md_bvh_steps(ref_md_bvh* s, int64_t steps) {
    const int32_t n = s->n;
    const double h = 0.5 * s->p.dt;
    for (int64_t k = 0; k < steps; ++k) {
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; ++i)
            for (int d = 0; d < 3; ++d) {
                s->v[3 * i + d] += h * s->f[3 * i + d] * s->im[i];
                s->x[3 * i + d] += s->p.dt * s->v[3 * i + d];
            }
        reflect(&s->p, n, s->x, s->v);
        ++s->done;
        if (s->rebuild > 0 && s->done % s->rebuild == 0) {
            int64_t st = build_half_list(s->x, n, s->rl, s->apl, s->order, &s->L);
            if (st < 0) return st;
        }
        forces_from_list(&s->p, n, s->x, s->q, &s->L, s->f, s->fth, s->nt);
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; ++i)
            for (int d = 0; d < 3; ++d) s->v[3 * i + d] += h * s->f[3 * i + d] * s->im[i];
    }
    return s->L.n;
}

void ref_md_bvh_get(const ref_md_bvh* s, double* x, double* v, double* f) {
    const size_t b = sizeof(double) * 3 * (size_t)s->n;
    if (x) memcpy(x, s->x, b);
    if (v) memcpy(v, s->v, b);
    if (f) memcpy(f, s->f, b);
}

void ref_md_bvh_destroy(ref_md_bvh* s) {
    if (!s) return;
    free(s->x); free(s->v); free(s->f); free(s->q); free(s->im); free(s->fth);
    free(s->L.i); free(s->L.j);
    free(s);
}

/* ------------------------------------------------------ synthetic inputs */

/* The benchmark workloads' seeded inputs, generated here so that the CPU
 * baseline needs nothing but this library: a splitmix64 stream (Steele, Lea
 * and Flood 2014), uniforms from its top 53 bits, normals by Box-Muller (one
 * value per pair of uniforms), positions by random sequential addition with a
 * minimum separation over a cell grid, charges +1 / -1 half each shuffled by
 * Fisher-Yates.  They match the GPU library's host generators bit for bit
 * (checked by the test suite). */
typedef struct { uint64_t s; } sm64;

static uint64_t sm64_next(sm64* g) {
    uint64_t z = (g->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double sm64_uniform(sm64* g) { return (double)(sm64_next(g) >> 11) * 0x1.0p-53; }

static double sm64_normal(sm64* g) {
    double u1 = sm64_uniform(g);
    double u2 = sm64_uniform(g);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

int ref_synth_uniform(uint64_t seed, int32_t n, double lo, double side, float* xyz) {
    if (!xyz || n < 0) return REF_ERR_ARG;
    sm64 g = {seed};
    for (int64_t k = 0; k < 3LL * n; ++k) xyz[k] = (float)(lo + side * sm64_uniform(&g));
    return 0;
}

int ref_synth_uniform_mindist(uint64_t seed, int32_t n, double side, double dmin, double* xyz) {
    if (!xyz || n < 0 || !(side > 0) || !(dmin >= 0)) return REF_ERR_ARG;
    sm64 g = {seed};
    int nc = dmin > 0 ? (int)floor(side / dmin) : 1;
    if (nc < 1) nc = 1;
    if (nc > 1024) nc = 1024;
    const double cs = side / nc;
    const size_t ncell = (size_t)nc * nc * nc;
    int32_t* head = (int32_t*)malloc(sizeof(int32_t) * ncell);
    int32_t* next = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    if (!head || !next) { free(head); free(next); return REF_ERR_NOMEM; }
    for (size_t c = 0; c < ncell; ++c) head[c] = -1;
    const double d2 = dmin * dmin;
    int status = 0;
    for (int32_t i = 0; i < n && status == 0; ++i) {
        int placed = 0;
        for (int attempt = 0; attempt < 100000 && !placed; ++attempt) {
            double p[3];
            int ci[3];
            for (int d = 0; d < 3; ++d) {
                p[d] = side * sm64_uniform(&g);
                int c = (int)(p[d] / cs);
                ci[d] = c < nc - 1 ? c : nc - 1;
            }
            int ok = 1;
            for (int oz = -1; oz <= 1 && ok; ++oz)
                for (int oy = -1; oy <= 1 && ok; ++oy)
                    for (int ox = -1; ox <= 1 && ok; ++ox) {
                        int X = ci[0] + ox, Y = ci[1] + oy, Z = ci[2] + oz;
                        if (X < 0 || Y < 0 || Z < 0 || X >= nc || Y >= nc || Z >= nc) continue;
                        for (int32_t j = head[((size_t)Z * nc + Y) * nc + X]; j >= 0; j = next[j]) {
                            double dx = p[0] - xyz[3 * (size_t)j], dy = p[1] - xyz[3 * (size_t)j + 1],
                                   dz = p[2] - xyz[3 * (size_t)j + 2];
                            if (dx * dx + dy * dy + dz * dz < d2) { ok = 0; break; }
                        }
                    }
            if (!ok) continue;
            for (int d = 0; d < 3; ++d) xyz[3 * (size_t)i + d] = p[d];
            size_t cell = ((size_t)ci[2] * nc + ci[1]) * nc + ci[0];
            next[i] = head[cell];
            head[cell] = i;
            placed = 1;
        }
        if (!placed) status = REF_ERR_ARG;
    }
    free(head);
    free(next);
    return status;
}

int ref_synth_normal(uint64_t seed, int64_t count, double s, double* out) {
    if (!out || count < 0) return REF_ERR_ARG;
    sm64 g = {seed};
    for (int64_t k = 0; k < count; ++k) out[k] = s * sm64_normal(&g);
    return 0;
}

int ref_synth_charges(uint64_t seed, int32_t n, double* q) {
    if (!q || n < 0 || (n & 1)) return REF_ERR_ARG;
    sm64 g = {seed};
    for (int32_t i = 0; i < n; ++i) q[i] = i < n / 2 ? 1.0 : -1.0;
    for (int32_t i = n - 1; i > 0; --i) {
        int32_t j = (int32_t)(sm64_next(&g) % (uint64_t)(i + 1));
        double t = q[i];
        q[i] = q[j];
        q[j] = t;
    }
    return 0;
}
