// nd_capi.cu -- the extern "C" boundary of libnaivegpu (declared in
// include/naivegpu.h): contexts, buffer management, status codes, the
// reference-shaped entry points and the seeded synthetic-input generators.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <set>
#include <vector>

#include "nd_internal.cuh"

struct nd_md;

// A context tracks its live engines: destroying the context releases their
// device state first and leaves the handles orphaned (every call on them then
// returns ND_ERR_ARG and nd_md_destroy only frees the handle), so the two may
// be destroyed in either order.
struct nd_adj;

struct nd_ctx {
    nd::Ctx c;
    std::set<nd_md*> engines;
    std::set<nd_adj*> adjoints;
};

struct nd_md {
    nd_ctx* ctx;
    nd::MDEngine* e;
};

struct nd_adj {
    nd_ctx* ctx;
    nd::AdjEngine* e;
};

static nd_md* md_register(nd_ctx* h, nd::MDEngine* e) {
    nd_md* md = new nd_md{h, e};
    h->engines.insert(md);
    return md;
}

static bool md_live(const nd_md* md) { return md && md->ctx && md->e; }

namespace nd {

nd_status cuda_fail(Ctx* c, cudaError_t e, const char* what) {
    c->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();  // clear a sticky-free error so later calls can proceed
    return e == cudaErrorMemoryAllocation ? ND_ERR_NOMEM : ND_ERR_CUDA;
}

nd_status check_launch(Ctx* c, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, what);
    return ND_OK;
}

nd_status ensure(Ctx* c, DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.p && b.bytes >= bytes) return ND_OK;
    if (c->no_alloc) {
        c->last_error = "scratch slice too small (no-allocation mode)";
        return ND_ERR_NOMEM;
    }
    if (b.p) {
        cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        cudaGetLastError();
        char msg[128];
        snprintf(msg, sizeof(msg), "cudaMalloc of %zu bytes", bytes);
        c->last_error = std::string(msg) + ": " + cudaGetErrorString(e);
        return ND_ERR_NOMEM;
    }
    b.bytes = bytes;
    return ND_OK;
}

static const char* status_text(nd_status st) {
    switch (st) {
        case ND_OK: return "ok";
        case ND_NEED_REALLOC: return "output buffer too small";
        case ND_ERR_ARG: return "invalid argument";
        case ND_ERR_SPEC: return "invalid BVH specification";
        case ND_ERR_NONFINITE: return "non-finite coordinate";
        case ND_ERR_RANGE: return "coordinate out of Int32 range after quantisation";
        case ND_ERR_CUDA: return "CUDA runtime error";
        case ND_ERR_NOMEM: return "device allocation failed";
        case ND_ERR_INTERNAL: return "device consistency check failed";
        case ND_ERR_OVERFLOW: return "neighbour list capacity exceeded";
        case ND_ERR_NODEVICE: return "no such CUDA device";
        default: return "unknown status";
    }
}

nd_status sync_and_check(Ctx* c, const char* what) {
    cudaError_t e = cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int32_t) * kErrWords,
                                    cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, what);
    if (c->h_err[0] != 0) {
        nd_status st = c->h_err[0];
        char msg[256];
        snprintf(msg, sizeof(msg), "%s: %s (item %d)", what, status_text(st), c->h_err[1]);
        c->last_error = msg;
        cudaMemsetAsync(c->d_err, 0, sizeof(int32_t) * kErrWords, c->stream);
        cudaStreamSynchronize(c->stream);
        return st;
    }
    return ND_OK;
}

static nd_status set_device(Ctx* c) {
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
    return ND_OK;
}

static void free_buf(DevBuf& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

static nd_status spec_ok(const nd_bvh_spec* s) {
    if (!s) return ND_ERR_ARG;
    if (s->atomsperleaf <= 0 || s->atom_count <= 0) return ND_ERR_SPEC;
    if (s->atom_count % s->atomsperleaf != 0) return ND_ERR_SPEC;
    int32_t nl = s->atom_count / s->atomsperleaf;
    if (nl < 2 || s->leaves_count != nl || s->branches_count != nl - 1) return ND_ERR_SPEC;
    return ND_OK;
}

// Upload host positions and build the tree on the context's scratch buffers.
static nd_status tree_from_host(Ctx* c, const float* xyz, const nd_bvh_spec* s, int32_t order,
                                int32_t boxes, int64_t nkeys, bool overwrite_root,
                                TreeBuffers* t) {
    const int32_t n = s->atom_count;
    nd_status st = ensure(c, c->xyz, 3 * sizeof(float) * (size_t)n);
    if (st) return st;
    cudaError_t e = cudaMemcpyAsync(c->xyz.p, xyz, 3 * sizeof(float) * (size_t)n,
                                    cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "position upload");
    return build_tree(c, (const float*)c->xyz.p, n, s->neighbor_distance, s->atomsperleaf, order,
                      boxes, nkeys, overwrite_root, t);
}

static nd_status pairs_from_tree(Ctx* c, const TreeBuffers& t, const nd_bvh_spec* s,
                                 int32_t mode, int kind, bool host, int32_t* pi, int32_t* pj,
                                 float* pd, int64_t capacity, int64_t* count, int32_t criterion);

nd_status pairs_common(Ctx* c, const nd_bvh_spec* s, int32_t order, int32_t mode, int kind,
                       const float* xyz, bool host, int32_t* pi, int32_t* pj, float* pd,
                       int64_t capacity, int64_t* count, int32_t criterion) {
    NvtxRange nv("nd leaf pairs");
    nd_status st = spec_ok(s);
    if (st) return st;
    if (criterion != ND_CRIT_SQUARED && criterion != ND_CRIT_SQRT) return ND_ERR_ARG;
    if (!xyz || !count || capacity < 0) return ND_ERR_ARG;
    if (capacity > 0 && (!pi || !pj || !pd)) return ND_ERR_ARG;
    if (order != ND_ORDER_REFERENCE && order != ND_ORDER_SPATIAL) return ND_ERR_ARG;
    if ((st = set_device(c))) return st;
    const int32_t n = s->atom_count, nL = s->leaves_count;
    const int32_t boxes = (kind == 0) ? ND_BOX_LEAF : ND_BOX_ATOM;
    if (kind == 0 && n - 1 < 2 * nL - 1) return ND_ERR_SPEC;  // leafTreeData needs apl >= 2
    TreeBuffers t;
    if (host) {
        st = tree_from_host(c, xyz, s, order, boxes, 2LL * nL - 1, false, &t);
    } else {
        st = build_tree(c, xyz, n, s->neighbor_distance, s->atomsperleaf, order, boxes,
                        2LL * nL - 1, false, &t);
    }
    if (st) return st;
    return pairs_from_tree(c, t, s, mode, kind, host, pi, pj, pd, capacity, count, criterion);
}

// Pair emission over a built tree (the second half of pairs_common).
static nd_status pairs_from_tree(Ctx* c, const TreeBuffers& t, const nd_bvh_spec* s,
                                 int32_t mode, int kind, bool host, int32_t* pi, int32_t* pj,
                                 float* pd, int64_t capacity, int64_t* count,
                                 int32_t criterion) {
    nd_status st;
    const float r = s->neighbor_distance;
    const float r2 = pair_threshold(r, criterion);
    int64_t total = 0;
    if (kind == 0 && mode == ND_PAIRS_UNORDERED && s->atomsperleaf == 4) {
        if (host) {
            int64_t devcap = (int64_t)(c->pairs_i.bytes / sizeof(int32_t));
            devcap = std::min(devcap, (int64_t)(c->pairs_d.bytes / sizeof(float)));
            if ((st = emit_unordered(c, t, r, r2, (int32_t*)c->pairs_i.p, (int32_t*)c->pairs_j.p,
                                     (float*)c->pairs_d.p, devcap, &total)))
                return st;
            *count = total;
            if (total > capacity) return ND_NEED_REALLOC;
            if (total > devcap) {
                if ((st = ensure(c, c->pairs_i, sizeof(int32_t) * (size_t)total))) return st;
                if ((st = ensure(c, c->pairs_j, sizeof(int32_t) * (size_t)total))) return st;
                if ((st = ensure(c, c->pairs_d, sizeof(float) * (size_t)total))) return st;
                int64_t again = 0;
                if ((st = emit_unordered(c, t, r, r2, (int32_t*)c->pairs_i.p, (int32_t*)c->pairs_j.p,
                                         (float*)c->pairs_d.p, total, &again)))
                    return st;
            }
        } else {
            if ((st = emit_unordered(c, t, r, r2, pi, pj, pd, capacity, &total))) return st;
            *count = total;
            return total > capacity ? ND_NEED_REALLOC : ND_OK;
        }
    } else {
        if ((st = count_pairs(c, t, r2, kind, &total))) return st;
        *count = total;
        if (total > capacity) return ND_NEED_REALLOC;
        if (total == 0) return ND_OK;
        if (host) {
            if ((st = ensure(c, c->pairs_i, sizeof(int32_t) * (size_t)total))) return st;
            if ((st = ensure(c, c->pairs_j, sizeof(int32_t) * (size_t)total))) return st;
            if ((st = ensure(c, c->pairs_d, sizeof(float) * (size_t)total))) return st;
            if ((st = write_pairs(c, t, r2, kind, (int32_t*)c->pairs_i.p, (int32_t*)c->pairs_j.p,
                                  (float*)c->pairs_d.p)))
                return st;
        } else {
            if ((st = write_pairs(c, t, r2, kind, pi, pj, pd))) return st;
            return sync_and_check(c, "pair write");
        }
    }
    // host copy-out
    if (total > 0) {
        cudaError_t e = cudaMemcpyAsync(pi, c->pairs_i.p, sizeof(int32_t) * (size_t)total,
                                        cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(pj, c->pairs_j.p, sizeof(int32_t) * (size_t)total,
                                cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(pd, c->pairs_d.p, sizeof(float) * (size_t)total,
                                cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "pair download");
    }
    return sync_and_check(c, "pairs");
}

// ------------------------------------------------------- synthetic inputs

struct SplitMix {
    uint64_t s;
    explicit SplitMix(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }  // [0, 1)
    double normal() {
        // Box-Muller, one value per call (the partner is discarded for simplicity)
        double u1 = uniform();
        double u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

}  // namespace nd

using nd::Ctx;

extern "C" {

nd_status nd_ctx_create(nd_ctx** out, int32_t device) {
    if (!out) return ND_ERR_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return ND_ERR_NODEVICE;
    }
    if (device < 0 || device >= count) return ND_ERR_NODEVICE;
    nd_ctx* h = new (std::nothrow) nd_ctx();
    if (!h) return ND_ERR_NOMEM;
    Ctx* c = &h->c;
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_err, sizeof(int32_t) * nd::kErrWords);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_err, sizeof(int32_t) * nd::kErrWords);
    if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(int32_t) * nd::kErrWords);
    if (e != cudaSuccess) {
        cudaGetLastError();
        nd_ctx_destroy(h);
        return e == cudaErrorMemoryAllocation ? ND_ERR_NOMEM : ND_ERR_CUDA;
    }
    *out = h;
    return ND_OK;
}

nd_status nd_ctx_destroy(nd_ctx* h) {
    if (!h) return ND_OK;
    Ctx* c = &h->c;
    cudaSetDevice(c->device);
    for (nd_md* md : h->engines) {
        nd::md_destroy(md->e);
        md->e = nullptr;
        md->ctx = nullptr;
    }
    h->engines.clear();
    for (nd_adj* a : h->adjoints) {
        nd::adj_destroy(a->e);
        a->e = nullptr;
        a->ctx = nullptr;
    }
    h->adjoints.clear();
    if (c->sim_cache) nd::md_destroy(c->sim_cache);
    c->sim_cache = nullptr;
    if (c->stream) cudaStreamSynchronize(c->stream);
    nd::DevBuf* bufs[] = {&c->xyz, &c->codes, &c->codes_alt, &c->perm, &c->perm_alt, &c->pos4,
                          &c->idx, &c->keys, &c->store, &c->hist, &c->counts, &c->offsets,
                          &c->partial, &c->pairs_i, &c->pairs_j, &c->pairs_d, &c->misc, &c->hash,
                          &c->leafpairs, &c->ranges, &c->tasks, &c->compat};
    for (nd::DevBuf* b : bufs) nd::free_buf(*b);
    if (c->d_err) cudaFree(c->d_err);
    if (c->h_err) cudaFreeHost(c->h_err);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete h;
    return ND_OK;
}

const char* nd_last_error(const nd_ctx* h) { return h ? h->c.last_error.c_str() : "no context"; }

const char* nd_status_string(nd_status st) { return nd::status_text(st); }

void* nd_ctx_stream(nd_ctx* h) { return h ? (void*)h->c.stream : nullptr; }

nd_status nd_ctx_device_name(const nd_ctx* h, char* buf, int32_t len) {
    if (!h || !buf || len <= 0) return ND_ERR_ARG;
    cudaDeviceProp prop{};
    cudaError_t e = cudaGetDeviceProperties(&prop, h->c.device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return ND_ERR_CUDA;
    }
    snprintf(buf, (size_t)len, "%s sm_%d%d x%d", prop.name, prop.major, prop.minor,
             prop.multiProcessorCount);
    return ND_OK;
}

nd_status nd_ctx_synchronize(nd_ctx* h) {
    if (!h) return ND_ERR_ARG;
    return nd::sync_and_check(&h->c, "synchronize");
}

int64_t nd_ctx_launch_count(const nd_ctx* h) { return h ? h->c.launches : 0; }

nd_status nd_bvh_spec_init(nd_bvh_spec* out, float r, int32_t n, int32_t apl) {
    if (!out) return ND_ERR_ARG;
    if (apl <= 0 || n <= 0 || n % apl != 0) return ND_ERR_SPEC;
    int32_t nl = n / apl;
    if (nl < 2) return ND_ERR_SPEC;
    out->neighbor_distance = r;
    out->atom_count = n;
    out->leaves_count = nl;
    out->branches_count = nl - 1;
    out->atomsperleaf = apl;
    return ND_OK;
}

nd_status nd_morton_codes_dev(nd_ctx* h, const float* xyz, int32_t n, int32_t order,
                              int32_t* codes) {
    if (!h || !xyz || !codes || n < 0) return ND_ERR_ARG;
    Ctx* c = &h->c;
    nd_status st = nd::set_device(c);
    if (st) return st;
    if ((st = nd::morton_codes(c, xyz, n, order, codes, nullptr))) return st;
    return nd::sync_and_check(c, "morton codes");
}

nd_status nd_sortperm_dev(nd_ctx* h, int32_t* codes, int32_t n, int32_t* perm) {
    if (!h || !codes || !perm || n < 0) return ND_ERR_ARG;
    Ctx* c = &h->c;
    nd_status st = nd::set_device(c);
    if (st) return st;
    // perm starts as the identity; the sort carries it along (stable)
    std::vector<int32_t> iota((size_t)n);
    for (int32_t i = 0; i < n; ++i) iota[i] = i;
    cudaError_t e = cudaMemcpyAsync(perm, iota.data(), sizeof(int32_t) * (size_t)n,
                                    cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return nd::cuda_fail(c, e, "perm init");
    if ((st = nd::radix_sort_pairs(c, (uint32_t*)codes, perm, n, 31))) return st;
    return nd::sync_and_check(c, "sortperm");
}

nd_status nd_tree(nd_ctx* h, const float* xyz, const nd_bvh_spec* s, int32_t order,
                  int32_t boxes, nd_gridkey* keys, int64_t nkeys, int32_t* index,
                  int32_t* morton_code, float* position, int32_t* perm) {
    if (!h || !xyz) return ND_ERR_ARG;
    Ctx* c = &h->c;
    nd_status st = nd::spec_ok(s);
    if (st) return st;
    if (order != ND_ORDER_REFERENCE && order != ND_ORDER_SPATIAL) return ND_ERR_ARG;
    if (boxes != ND_BOX_LEAF && boxes != ND_BOX_ATOM) return ND_ERR_ARG;
    const int32_t n = s->atom_count, nL = s->leaves_count;
    if (boxes == ND_BOX_LEAF && n - 1 < 2 * nL - 1) return ND_ERR_SPEC;
    if (keys && nkeys < 0) return ND_ERR_ARG;
    if ((st = nd::set_device(c))) return st;
    const int64_t need = std::max<int64_t>(2LL * nL - 1, boxes == ND_BOX_LEAF ? n - 1 : 0);
    nd::TreeBuffers t;
    if ((st = nd::tree_from_host(c, xyz, s, order, boxes, need, true, &t))) return st;
    std::vector<float4> pos4;
    cudaError_t e = cudaSuccess;
    if (keys && nkeys > 0) {
        int64_t k = std::min(nkeys, need);
        e = cudaMemcpyAsync(keys, t.keys, 32 * (size_t)k, cudaMemcpyDeviceToHost, c->stream);
        if (nkeys > k) memset(keys + k, 0, 32 * (size_t)(nkeys - k));
    }
    if (e == cudaSuccess && index)
        e = cudaMemcpyAsync(index, t.idx, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && morton_code)
        e = cudaMemcpyAsync(morton_code, t.codes, sizeof(int32_t) * (size_t)n,
                            cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && perm)
        e = cudaMemcpyAsync(perm, t.perm, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && position) {
        pos4.resize((size_t)n);
        e = cudaMemcpyAsync(pos4.data(), t.pos4, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToHost,
                            c->stream);
    }
    if (e != cudaSuccess) return nd::cuda_fail(c, e, "tree download");
    if ((st = nd::sync_and_check(c, "tree"))) return st;
    if (perm)
        for (int32_t i = 0; i < n; ++i) perm[i] += 1;  // 1-based, as Julia's sortperm
    if (position)
        for (int32_t i = 0; i < n; ++i) {
            position[3 * (size_t)i] = pos4[i].x;
            position[3 * (size_t)i + 1] = pos4[i].y;
            position[3 * (size_t)i + 2] = pos4[i].z;
        }
    return ND_OK;
}

nd_status nd_leaf_pairs(nd_ctx* h, const float* xyz, const nd_bvh_spec* s, int32_t order,
                        int32_t mode, int32_t* pi, int32_t* pj, float* pd, int64_t capacity,
                        int64_t* count) {
    if (!h) return ND_ERR_ARG;
    return nd::pairs_common(&h->c, s, order, mode, 0, xyz, true, pi, pj, pd, capacity, count);
}

nd_status nd_leaf_pairs_dev(nd_ctx* h, const float* xyz, const nd_bvh_spec* s, int32_t order,
                            int32_t mode, int32_t* pi, int32_t* pj, float* pd, int64_t capacity,
                            int64_t* count) {
    if (!h) return ND_ERR_ARG;
    return nd::pairs_common(&h->c, s, order, mode, 0, xyz, false, pi, pj, pd, capacity, count);
}

nd_status nd_leaf_pairs_refresh(nd_ctx* h, const float* xyz, const nd_bvh_spec* s,
                                const int32_t* index, const int32_t* morton_code, int32_t mode,
                                nd_gridkey* keys, int64_t nkeys, float* position, int32_t* pi,
                                int32_t* pj, float* pd, int64_t capacity, int64_t* count) {
    if (!h || !xyz || !index || !morton_code || !count || capacity < 0) return ND_ERR_ARG;
    if (capacity > 0 && (!pi || !pj || !pd)) return ND_ERR_ARG;
    if (keys && nkeys < 0) return ND_ERR_ARG;
    Ctx* c = &h->c;
    nd_status st = nd::spec_ok(s);
    if (st) return st;
    const int32_t n = s->atom_count, nL = s->leaves_count;
    if (n - 1 < 2 * nL - 1) return ND_ERR_SPEC;  // leafTreeData needs atomsperleaf >= 2
    if (mode != ND_PAIRS_ORDERED && mode != ND_PAIRS_UNORDERED) return ND_ERR_ARG;
    // the kept order must be a permutation and its codes ascending
    {
        std::vector<uint8_t> seen((size_t)n, 0);
        for (int32_t k = 0; k < n; ++k) {
            const int32_t v = index[k];
            if (v < 1 || v > n || seen[v - 1]) return ND_ERR_ARG;
            seen[v - 1] = 1;
            if (morton_code[k] < 0 || (k > 0 && morton_code[k] < morton_code[k - 1]))
                return ND_ERR_ARG;
        }
    }
    if ((st = nd::set_device(c))) return st;
    if ((st = nd::ensure(c, c->xyz, 3 * sizeof(float) * (size_t)n))) return st;
    if ((st = nd::ensure(c, c->perm_alt, sizeof(int32_t) * (size_t)n))) return st;
    if ((st = nd::ensure(c, c->codes, sizeof(int32_t) * (size_t)n))) return st;
    cudaError_t e = cudaMemcpyAsync(c->xyz.p, xyz, 3 * sizeof(float) * (size_t)n,
                                    cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->perm_alt.p, index, sizeof(int32_t) * (size_t)n,
                            cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->codes.p, morton_code, sizeof(int32_t) * (size_t)n,
                            cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return nd::cuda_fail(c, e, "refresh upload");
    const int64_t need = std::max<int64_t>(2LL * nL - 1, n - 1);
    nd::TreeBuffers t;
    if ((st = nd::build_tree_kept(c, (const float*)c->xyz.p, n, s->neighbor_distance,
                                  s->atomsperleaf, (const int32_t*)c->perm_alt.p,
                                  (const int32_t*)c->codes.p, need, &t)))
        return st;
    const nd_status pst = pairs_from_tree(c, t, s, mode, 0, true, pi, pj, pd, capacity, count,
                                          ND_CRIT_SQUARED);
    if (pst != ND_OK && pst != ND_NEED_REALLOC) return pst;
    // the kept tree with the new boxes (root box overwritten, as the reference
    // returns it) and the positions in the kept order
    nd::root_overwrite(c, t.keys, nL);
    std::vector<float4> pos4;
    if (keys && nkeys > 0) {
        const int64_t k = std::min(nkeys, need);
        e = cudaMemcpyAsync(keys, t.keys, 32 * (size_t)k, cudaMemcpyDeviceToHost, c->stream);
        if (nkeys > k) memset(keys + k, 0, 32 * (size_t)(nkeys - k));
    }
    if (e == cudaSuccess && position) {
        pos4.resize((size_t)n);
        e = cudaMemcpyAsync(pos4.data(), t.pos4, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToHost,
                            c->stream);
    }
    if (e != cudaSuccess) return nd::cuda_fail(c, e, "refresh download");
    if ((st = nd::sync_and_check(c, "refresh"))) return st;
    if (position)
        for (int32_t i = 0; i < n; ++i) {
            position[3 * (size_t)i] = pos4[i].x;
            position[3 * (size_t)i + 1] = pos4[i].y;
            position[3 * (size_t)i + 2] = pos4[i].z;
        }
    return pst;
}

nd_status nd_simd_leaf_pairs(nd_ctx* h, const float* xyz, const nd_bvh_spec* s, int32_t order,
                             int32_t mode, int32_t* pi, int32_t* pj, float* pd,
                             int64_t capacity, int64_t* count) {
    if (!h || !s) return ND_ERR_ARG;
    if (s->atomsperleaf != 4) return ND_ERR_SPEC;  // simdTreeData asserts atomsperleaf == 4
    return nd::pairs_common(&h->c, s, order, mode, 0, xyz, true, pi, pj, pd, capacity, count,
                            ND_CRIT_SQRT);
}

nd_status nd_atom_pairs(nd_ctx* h, const float* xyz, const nd_bvh_spec* s, int32_t order,
                        int32_t* pi, int32_t* pj, float* pd, int64_t capacity, int64_t* count) {
    if (!h) return ND_ERR_ARG;
    return nd::pairs_common(&h->c, s, order, ND_PAIRS_ORDERED, 1, xyz, true, pi, pj, pd, capacity,
                            count);
}

nd_status nd_pair_hash_dev(nd_ctx* h, const int32_t* pi, const int32_t* pj, const float* pd,
                           int64_t np, uint64_t hash[2]) {
    if (!h || !hash || np < 0 || (np > 0 && (!pi || !pj || !pd))) return ND_ERR_ARG;
    Ctx* c = &h->c;
    nd_status st = nd::set_device(c);
    if (st) return st;
    return nd::pair_hash(c, pi, pj, pd, np, hash);
}

nd_status nd_forces_pairs(nd_ctx* h, const nd_md_params* p, int32_t n, const double* x,
                          const double* q, const int32_t* pi, const int32_t* pj, int64_t npairs,
                          float* force, double* energy) {
    if (!h) return ND_ERR_ARG;
    Ctx* c = &h->c;
    nd_status st = nd::set_device(c);
    if (st) return st;
    return nd::forces_pairs(c, p, n, x, q, pi, pj, npairs, force, energy);
}

nd_status nd_compat_force_lennardjones(nd_ctx* h, int32_t n, const int32_t* pi,
                                       const int32_t* pj, const float* pd, int64_t npairs,
                                       float* force) {
    if (!h) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    return nd::compat_forces(&h->c, 0, n, pi, pj, pd, npairs, nullptr, force);
}

nd_status nd_compat_force_coulomb(nd_ctx* h, int32_t n, const int32_t* pi, const int32_t* pj,
                                  const float* pd, int64_t npairs, const float* charge,
                                  float* force) {
    if (!h) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    return nd::compat_forces(&h->c, 1, n, pi, pj, pd, npairs, charge, force);
}

nd_status nd_collect_objects(nd_ctx* h, const nd_collector* collector, uint64_t seed,
                             float* position, float* velocity, float* mass, float* charge,
                             int64_t* pruned) {
    if (!h) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    return nd::collect_objects(&h->c, collector, seed, position, velocity, mass, charge, pruned);
}

nd_status nd_compat_simulate(nd_ctx* h, const nd_compat_sim* spec, int32_t n, float* position,
                             float* velocity, float* force, const float* mass,
                             const float* charge, float* poslog) {
    if (!h) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    return nd::compat_simulate(&h->c, spec, n, position, velocity, force, mass, charge, poslog);
}

nd_status nd_forces(nd_ctx* h, const nd_md_params* p, int32_t n, const double* x,
                    const double* q, float* force, double* energy) {
    if (!h || !p || !x || n <= 0) return ND_ERR_ARG;
    Ctx* c = &h->c;
    nd_status st = nd::set_device(c);
    if (st) return st;
    nd_md_params pp = *p;
    if (pp.rebuild_every <= 0) pp.rebuild_every = 1;
    if (!(pp.dt > 0)) pp.dt = 1.0;
    std::vector<double> v0(3 * (size_t)n, 0.0);
    nd::MDEngine* m = nullptr;
    if ((st = nd::md_create(c, &pp, n, x, v0.data(), q, nullptr, true, false, &m))) return st;
    st = nd::md_get(m, nullptr, nullptr, force, true);
    if (st == ND_OK && energy) {
        double pot = 0.0;
        st = nd::md_energy(m, &pot, nullptr);
        *energy = pot;
    }
    if (st) c->last_error = nd::md_last_error(m);
    nd::md_destroy(m);
    return st;
}

nd_status nd_md_create(nd_ctx* h, const nd_md_params* p, int32_t n, const double* x,
                       const double* v, const double* q, const double* m, nd_md** out) {
    if (!h || !out) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    nd::MDEngine* e = nullptr;
    if ((st = nd::md_create(&h->c, p, n, x, v, q, m, true, true, &e))) return st;
    *out = md_register(h, e);
    return ND_OK;
}

nd_status nd_md_create_dev(nd_ctx* h, const nd_md_params* p, int32_t n, const double* x,
                           const double* v, const double* q, const double* m, nd_md** out) {
    if (!h || !out) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    nd::MDEngine* e = nullptr;
    if ((st = nd::md_create(&h->c, p, n, x, v, q, m, false, true, &e))) return st;
    *out = md_register(h, e);
    return ND_OK;
}

nd_status nd_batch_create(nd_ctx* h, const nd_md_params* p, int32_t nsys, const nd_system* sys,
                          const double* x, const double* v, const double* q, const double* m,
                          nd_md** out) {
    if (!h || !out) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    nd::MDEngine* e = nullptr;
    if ((st = nd::md_create_batch(&h->c, p, nsys, sys, x, v, q, m, true, &e))) return st;
    *out = md_register(h, e);
    return ND_OK;
}

nd_status nd_batch_create_dev(nd_ctx* h, const nd_md_params* p, int32_t nsys,
                              const nd_system* sys, const double* x, const double* v,
                              const double* q, const double* m, nd_md** out) {
    if (!h || !out) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    nd::MDEngine* e = nullptr;
    if ((st = nd::md_create_batch(&h->c, p, nsys, sys, x, v, q, m, false, &e))) return st;
    *out = md_register(h, e);
    return ND_OK;
}

nd_status nd_batch_energies(nd_md* md, double* potential, double* kinetic) {
    if (!md_live(md)) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    nd_status st = nd::md_energies(md->e, potential, kinetic);
    if (st) md->ctx->c.last_error = nd::md_last_error(md->e);
    return st;
}

nd_status nd_md_autotune(nd_ctx* h, const nd_md_params* p, int32_t n, int32_t nsys,
                         const nd_system* sys, const double* x, const double* v, const double* q,
                         const double* m, int32_t trial_steps, nd_md_params* best,
                         double* seconds_per_step) {
    if (!h) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    return nd::md_autotune(&h->c, p, n, nsys, sys, x, v, q, m, trial_steps, best,
                           seconds_per_step);
}

nd_status nd_md_destroy(nd_md* md) {
    if (!md) return ND_OK;
    if (md_live(md)) {
        nd::set_device(&md->ctx->c);
        md->ctx->engines.erase(md);
        nd::md_destroy(md->e);
    }
    delete md;
    return ND_OK;
}

static nd_status md_wrap(nd_md* md, nd_status st) {
    if (st) md->ctx->c.last_error = nd::md_last_error(md->e);
    return st;
}

nd_status nd_md_run(nd_md* md, int64_t steps) {
    if (!md_live(md) || steps < 0) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    return md_wrap(md, nd::md_run(md->e, steps));
}

nd_status nd_md_sync(nd_md* md) {
    if (!md_live(md)) return ND_ERR_ARG;
    return md_wrap(md, nd::md_sync(md->e));
}

nd_status nd_md_get(nd_md* md, double* x, double* v, float* f) {
    if (!md_live(md)) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    return md_wrap(md, nd::md_get(md->e, x, v, f, true));
}

nd_status nd_md_get_dev(nd_md* md, double* x, double* v, float* f) {
    if (!md_live(md)) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    return md_wrap(md, nd::md_get(md->e, x, v, f, false));
}

nd_status nd_md_energy(nd_md* md, double* potential, double* kinetic) {
    if (!md_live(md)) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    return md_wrap(md, nd::md_energy(md->e, potential, kinetic));
}

nd_status nd_md_stats(nd_md* md, int64_t* steps, int64_t* rebuilds, int64_t* list_pairs,
                      int32_t* capacity) {
    if (!md_live(md)) return ND_ERR_ARG;
    return md_wrap(md, nd::md_stats(md->e, steps, rebuilds, list_pairs, capacity));
}

nd_status nd_md_diagnostics(nd_md* md, nd_md_diag* out) {
    if (!md_live(md) || !out) return ND_ERR_ARG;
    return md_wrap(md, nd::md_diagnostics(md->e, out));
}

nd_status nd_md_list_pairs(nd_md* md, int32_t* pi, int32_t* pj, uint8_t* near,
                           int64_t capacity, int64_t* count) {
    if (!md_live(md) || capacity < 0) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    return md_wrap(md, nd::md_list_pairs(md->e, pi, pj, near, capacity, count));
}

nd_status nd_md_step_times(nd_md* md, int32_t steps, float* ms) {
    if (!md_live(md)) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    return md_wrap(md, nd::md_step_times(md->e, steps, ms));
}

nd_status nd_md_set_thermostat(nd_md* md, double temperature, double gamma, int32_t every) {
    if (!md_live(md)) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    return md_wrap(md, nd::md_set_thermostat(md->e, temperature, gamma, every));
}

nd_status nd_md_set_log(nd_md* md, int32_t every, int32_t frames) {
    if (!md_live(md)) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    return md_wrap(md, nd::md_set_log(md->e, every, frames));
}

nd_status nd_md_log_count(nd_md* md, int64_t* count) {
    if (!md_live(md) || !count) return ND_ERR_ARG;
    return md_wrap(md, nd::md_log_count(md->e, count));
}

nd_status nd_md_log_read(nd_md* md, int64_t first, int64_t nframes, double* out) {
    if (!md_live(md) || (nframes > 0 && !out)) return ND_ERR_ARG;
    nd::set_device(&md->ctx->c);
    return md_wrap(md, nd::md_log_read(md->e, first, nframes, out));
}

int64_t nd_md_launches_per_run(nd_md* md, int64_t steps) {
    return md_live(md) ? nd::md_launches_per_run(md->e, steps) : 0;
}

nd_status nd_simulate(nd_ctx* h, const nd_md_params* p, int32_t n, double* x, double* v,
                      float* f, const double* q, const double* m, int64_t steps) {
    nd::NvtxRange nv("nd simulate");
    if (!h || !p || !x || !v || steps < 0) return ND_ERR_ARG;
    Ctx* c = &h->c;
    nd_status st = nd::set_device(c);
    if (st) return st;
    // The context keeps the engine of its last call: a call with the same size
    // and parameters re-uses its buffers and captured graphs.
    nd::MDEngine* e = c->sim_cache;
    bool fresh = !nd::md_compatible(e, p, n, q != nullptr, m != nullptr);
    if (!fresh) {
        st = nd::md_reset(e, x, v, q, m, true);
        if (st == ND_ERR_OVERFLOW) fresh = true;
        else if (st) { c->last_error = nd::md_last_error(e); return st; }
    }
    if (fresh) {
        if (e) nd::md_destroy(e);
        c->sim_cache = nullptr;
        if ((st = nd::md_create(c, p, n, x, v, q, m, true, true, &e))) return st;
        c->sim_cache = e;
    }
    st = nd::md_run(e, steps);
    if (st == ND_OK) st = nd::md_get(e, x, v, f, true);
    if (st) {
        c->last_error = nd::md_last_error(e);
        nd::md_destroy(e);
        c->sim_cache = nullptr;
    }
    return st;
}

nd_status nd_simulate_diagnostics(nd_ctx* h, nd_md_diag* out) {
    if (!h || !out || !h->c.sim_cache) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    return nd::md_diagnostics(h->c.sim_cache, out);
}

// ------------------------------------------------------------------ adjoint

static bool adj_live(const nd_adj* a) { return a && a->ctx && a->e; }

static nd_status adj_wrap(nd_adj* a, nd_status st) {
    if (st) a->ctx->c.last_error = nd::adj_last_error(a->e);
    return st;
}

nd_status nd_adj_create(nd_ctx* h, const nd_md_params* p, int32_t n, const double* x0,
                        const double* v0, const double* q, const double* m,
                        const nd_adj_spec* spec, nd_adj** out) {
    if (!h || !out) return ND_ERR_ARG;
    nd_status st = nd::set_device(&h->c);
    if (st) return st;
    nd::AdjEngine* e = nullptr;
    if ((st = nd::adj_create(&h->c, p, n, x0, v0, q, m, spec, &e))) return st;
    nd_adj* a = new nd_adj{h, e};
    h->adjoints.insert(a);
    *out = a;
    return ND_OK;
}

nd_status nd_adj_destroy(nd_adj* a) {
    if (!a) return ND_OK;
    if (adj_live(a)) {
        nd::set_device(&a->ctx->c);
        a->ctx->adjoints.erase(a);
        nd::adj_destroy(a->e);
    }
    delete a;
    return ND_OK;
}

nd_status nd_adj_set_params(nd_adj* a, double sigma, double epsilon) {
    if (!adj_live(a)) return ND_ERR_ARG;
    return adj_wrap(a, nd::adj_set_params(a->e, sigma, epsilon));
}

nd_status nd_adj_set_target(nd_adj* a, const double* target) {
    if (!adj_live(a)) return ND_ERR_ARG;
    nd::set_device(&a->ctx->c);
    return adj_wrap(a, nd::adj_set_target(a->e, target));
}

nd_status nd_adj_forward(nd_adj* a, double* hist, double* loss) {
    if (!adj_live(a)) return ND_ERR_ARG;
    nd::set_device(&a->ctx->c);
    return adj_wrap(a, nd::adj_forward(a->e, hist, loss));
}

nd_status nd_adj_backward(nd_adj* a, double* dx0, double* dv0, double* dsigma,
                          double* depsilon) {
    if (!adj_live(a)) return ND_ERR_ARG;
    nd::set_device(&a->ctx->c);
    return adj_wrap(a, nd::adj_backward(a->e, dx0, dv0, dsigma, depsilon));
}

nd_status nd_adj_final(nd_adj* a, double* x) {
    if (!adj_live(a) || !x) return ND_ERR_ARG;
    nd::set_device(&a->ctx->c);
    return adj_wrap(a, nd::adj_final(a->e, x));
}

nd_status nd_adj_times(nd_adj* a, float* forward_ms, float* backward_ms) {
    if (!adj_live(a)) return ND_ERR_ARG;
    return adj_wrap(a, nd::adj_times(a->e, forward_ms, backward_ms));
}

// ------------------------------------------------------------ synthetic inputs

nd_status nd_synth_uniform(uint64_t seed, int32_t n, double lo, double side, float* xyz) {
    if (!xyz || n < 0) return ND_ERR_ARG;
    nd::SplitMix g(seed);
    for (int64_t k = 0; k < 3LL * n; ++k) xyz[k] = (float)(lo + side * g.uniform());
    return ND_OK;
}

nd_status nd_synth_uniform_mindist(uint64_t seed, int32_t n, double side, double dmin,
                                   double* xyz) {
    if (!xyz || n < 0 || !(side > 0) || !(dmin >= 0)) return ND_ERR_ARG;
    nd::SplitMix g(seed);
    int nc = dmin > 0 ? (int)std::floor(side / dmin) : 1;
    nc = std::max(1, std::min(nc, 1024));
    const double cs = side / nc;
    std::vector<int32_t> head((size_t)nc * nc * nc, -1), next((size_t)n, -1);
    const double d2 = dmin * dmin;
    for (int32_t i = 0; i < n; ++i) {
        bool placed = false;
        for (int attempt = 0; attempt < 100000 && !placed; ++attempt) {
            double p[3];
            int ci[3];
            for (int d = 0; d < 3; ++d) {
                p[d] = side * g.uniform();
                ci[d] = std::min(nc - 1, (int)(p[d] / cs));
            }
            bool ok = true;
            for (int oz = -1; oz <= 1 && ok; ++oz)
                for (int oy = -1; oy <= 1 && ok; ++oy)
                    for (int ox = -1; ox <= 1 && ok; ++ox) {
                        int X = ci[0] + ox, Y = ci[1] + oy, Z = ci[2] + oz;
                        if (X < 0 || Y < 0 || Z < 0 || X >= nc || Y >= nc || Z >= nc) continue;
                        for (int32_t j = head[((size_t)Z * nc + Y) * nc + X]; j >= 0; j = next[j]) {
                            double dx = p[0] - xyz[3 * (size_t)j], dy = p[1] - xyz[3 * (size_t)j + 1],
                                   dz = p[2] - xyz[3 * (size_t)j + 2];
                            if (dx * dx + dy * dy + dz * dz < d2) { ok = false; break; }
                        }
                    }
            if (!ok) continue;
            for (int d = 0; d < 3; ++d) xyz[3 * (size_t)i + d] = p[d];
            size_t cell = ((size_t)ci[2] * nc + ci[1]) * nc + ci[0];
            next[i] = head[cell];
            head[cell] = i;
            placed = true;
        }
        if (!placed) return ND_ERR_ARG;  // too dense for this minimum distance
    }
    return ND_OK;
}

nd_status nd_synth_clusters(uint64_t seed, int32_t n, int32_t nclusters, double side,
                            double smin, double smax, float* xyz) {
    if (!xyz || n < 0 || nclusters <= 0 || n % nclusters != 0) return ND_ERR_ARG;
    nd::SplitMix g(seed);
    const int32_t per = n / nclusters;
    for (int32_t c = 0; c < nclusters; ++c) {
        double ctr[3] = {side * g.uniform(), side * g.uniform(), side * g.uniform()};
        double sg = smin + (smax - smin) * g.uniform();
        for (int32_t k = 0; k < per; ++k) {
            size_t a = (size_t)c * per + k;
            for (int d = 0; d < 3; ++d) xyz[3 * a + d] = (float)(ctr[d] + sg * g.normal());
        }
    }
    return ND_OK;
}

nd_status nd_synth_normal(uint64_t seed, int64_t count, double s, double* out) {
    if (!out || count < 0) return ND_ERR_ARG;
    nd::SplitMix g(seed);
    for (int64_t k = 0; k < count; ++k) out[k] = s * g.normal();
    return ND_OK;
}

nd_status nd_synth_charges(uint64_t seed, int32_t n, double* q) {
    if (!q || n < 0 || (n & 1)) return ND_ERR_ARG;
    nd::SplitMix g(seed);
    for (int32_t i = 0; i < n; ++i) q[i] = i < n / 2 ? 1.0 : -1.0;
    for (int32_t i = n - 1; i > 0; --i) {
        int32_t j = (int32_t)(g.next() % (uint64_t)(i + 1));
        std::swap(q[i], q[j]);
    }
    return ND_OK;
}

}  // extern "C"
